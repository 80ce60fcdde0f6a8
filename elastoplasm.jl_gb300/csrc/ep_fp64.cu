// ep_fp64.cu -- the FP64 drop-in MPM step ("oracle order").
//
// Compiled with -fmad=false: every product and sum is rounded separately, as
// in the reference's Julia code, and every nodal sum is accumulated in
// ascending point order (the order of the reference's serial @atomic scatter),
// so this step reproduces the CPU restatement bit for bit.  Scatter-type
// transfers are therefore gathers: each node walks the sorted list of the
// points whose stencil holds it.
//
// Kernel (reference it implements)                               launch shape
//   k_bin64      p2e2n + ϕ∂ϕ tables + transform τ/J               point
//                (tplgy.jl:43-96, basis/*.jl, p2n.jl:12-21)
//   k_count_nodes / k_place_nodes / segsort   node -> point lists node / point
//   k_p2g64      std/tpic_{2,3}d_p2n (p2n.jl:135-268)            node
//   k_solve64    euler (solve.jl:14-40)                           node
//   k_g2p64      picflip_n2p (n2p.jl:14-40)                       point
//   k_augm64     augm_momentum + augm_velocity (augm.jl:13-53)    node
//   k_deform64   finite/infinitesimal_deform + domain             point
//                (deform.jl:1-44, domain.jl:1-52)
//   k_dJ64       ΔJn + ΔJs (volumetric.jl:1-22)                   node
//   k_elast64    ΔJp + elast (+ return map without nonlocal)      point
//                (volumetric.jl:23-36, elast.jl:45-80, DP.jl, J2.jl)
//   k_nonlocal64 nonlocal p->q / p<-q (nonlocal.jl:18-47)         warp per point
//   k_retmap64   finite/infinitesimal DP/J2                       point
#include <climits>

#include "../../include/epgpu.h"
#include "ep_internal.h"

namespace ep {

#define EP_ACTIVE(ctl) \
    if (!(ctl)->active) return

__device__ __forceinline__ double SHget(const P64& P, int np, int p, int d, int o, int c) {
    return P.SH[(size_t)((d * 4 + o) * 2 + c) * np + p];
}

__device__ __forceinline__ void atomic_max_abs(unsigned long long* a, double v) {
    atomicMax(a, (unsigned long long)__double_as_longlong(fabs(v)));
}

// shape value N and gradient of slot offsets o for point p (products as in bsmpm_{2,3}d)
template <int D>
__device__ __forceinline__ void shape_at(const P64& P, int np, int p, const int* o, double* N) {
    double f[3], g[3];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        f[d] = SHget(P, np, p, d, o[d], 0);
        g[d] = SHget(P, np, p, d, o[d], 1);
    }
    if (D == 2) {
        N[0] = f[0] * f[1];
        N[1] = g[0] * f[1];
        N[2] = f[0] * g[1];
    } else {
        N[0] = f[0] * f[1] * f[2];
        N[1] = g[0] * f[1] * f[2];
        N[2] = f[0] * g[1] * f[2];
        N[3] = f[0] * f[1] * g[2];
    }
}

// ---------------------------------------------------------------------------
template <int D, int BASIS>
__global__ void k_bin64(Cfg cf, Geo g, Ctl* ctl, P64 P, int* cell_count) {
    EP_ACTIVE(ctl);
    const int np = P.np;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    double xp[3];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        xp[d] = P.x[d][p];
        P.xo[d][p] = xp[d];
    }
    int e[3];
    int c = cell_index<D>(xp, g, e);
    P.p2e[p] = c;
    if (c < 0) {
        set_err(ctl, EP_ERR_NONFINITE, p);
        return;
    }
    atomicAdd(&cell_count[c], 1);
    if (cf.deform == EP_DEFORM_FINITE) {
        const int NS = D == 2 ? 3 : 6;
        double J = P.J[p];
#pragma unroll
        for (int s = 0; s < NS; ++s) P.sig[s][p] = P.tau[s][p] / J;
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
#pragma unroll
        for (int o = 0; o < 4; ++o) {
            int idx = e[d] - 1 + o;
            double f = 0.0, df = 0.0;
            if (idx >= 0 && idx < g.nno[d]) {
                double xn = g.ax[d][idx];
                if (BASIS == EP_BASIS_BSMPM) {
                    int cls = g.cls[d][idx];
                    if (cls == BS_INVALID) set_err(ctl, EP_ERR_INVALID_POSITION, p);
                    double xi = (xp[d] - xn) / g.h[d];
                    bspline(cls, xi, g.h[d], &f, &df);
                } else if (BASIS == EP_BASIS_GIMPM) {
                    gimp(xp[d] - xn, g.h[d], P.l[d][p], &f, &df);
                } else {
                    hat(xp[d] - xn, g.h[d], &f, &df);
                }
            }
            P.SH[(size_t)((d * 4 + o) * 2 + 0) * np + p] = f;
            P.SH[(size_t)((d * 4 + o) * 2 + 1) * np + p] = df;
        }
    }
    if (cf.trsfr == EP_TRSFR_APIC) {
        // Dij_nd (shpfun/misc.jl:15-28): D = N δ δᵀ of the last existing stencil node (it is
        // assigned node by node), then the step's B D⁻¹ (p2n.jl:221-226)
        const int NN = D == 2 ? 16 : 64;
        for (int s = NN - 1; s >= 0; --s) {
            int o[3], i[3];
            slot_offsets<D>(s, o);
            bool ok = true;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                i[d] = e[d] - 1 + o[d];
                ok = ok && i[d] >= 0 && i[d] < g.nno[d];
            }
            if (!ok) continue;
            double N[4], dl[3], Dm[D * D], Bp[D * D], C[D * D];
            shape_at<D>(P, np, p, o, N);
#pragma unroll
            for (int d = 0; d < D; ++d) dl[d] = g.ax[d][i[d]] - xp[d];
#pragma unroll
            for (int b = 0; b < D; ++b)
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    Dm[a + D * b] = N[0] * (dl[a] * dl[b]);
                    P.Dm[a + D * b][p] = Dm[a + D * b];
                    Bp[a + D * b] = P.B[a + D * b][p];
                }
            apic_bdinv<D>(Bp, Dm, C);
#pragma unroll
            for (int k = 0; k < D * D; ++k) P.BD[k][p] = C[k];
            break;
        }
    }
}

// number of points whose stencil holds each node: sum of the counts of the
// cells e with e_d in [i_d-2, i_d+1]
template <int D>
__global__ void k_count_nodes(Geo g, const Ctl* ctl, const int* __restrict__ cell_count, int* node_count) {
    EP_ACTIVE(ctl);
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nnode) return;
    int i[3];
    node_coords<D>(n, g, i);
    int lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        lo[d] = max(i[d] - 2, 0);
        hi[d] = min(i[d] + 1, g.nel[d] - 1);
    }
    int s = 0;
    if (D == 2) {
        for (int a = lo[0]; a <= hi[0]; ++a)
            for (int b = lo[1]; b <= hi[1]; ++b) s += cell_count[b + g.nel[1] * a];
    } else {
        for (int k = lo[1]; k <= hi[1]; ++k)
            for (int a = lo[0]; a <= hi[0]; ++a)
                for (int b = lo[2]; b <= hi[2]; ++b) s += cell_count[b + g.nel[2] * a + g.nel[2] * g.nel[0] * k];
    }
    node_count[n] = s;
}

template <int D>
__global__ void k_place_nodes(Geo g, const Ctl* ctl, const int* __restrict__ p2e, int np,
                              const int* __restrict__ node_start, int* cursor, int* node_list) {
    EP_ACTIVE(ctl);
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    int c = p2e[p];
    if (c < 0) return;
    int e[3];
    cell_coords<D>(c, g, e);
    const int NN = D == 2 ? 16 : 64;
    for (int s = 0; s < NN; ++s) {
        int o[3], i[3];
        slot_offsets<D>(s, o);
        bool ok = true;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            i[d] = e[d] - 1 + o[d];
            ok = ok && i[d] >= 0 && i[d] < g.nno[d];
        }
        if (!ok) continue;
        int n = node_id<D>(i, g);
        int k = atomicAdd(&cursor[n], 1);
        int pos = node_start[n] + k;
        if (pos < node_start[n + 1]) node_list[pos] = p;    // never taken unless the scan is corrupt
        else set_err(const_cast<Ctl*>(ctl), EP_ERR_CUDA, p);
    }
}

// offsets of node i inside the stencil of point p
template <int D>
__device__ __forceinline__ void offsets_of(const Geo& g, const int* i, int cell, int* o) {
    int e[3];
    cell_coords<D>(cell, g, e);
#pragma unroll
    for (int d = 0; d < D; ++d) o[d] = i[d] - e[d] + 1;
}

// ---------------------------------------------------------------------------
// P2G: m, p, f for one node, contributions in ascending point order.
template <int D>
__global__ void k_p2g64(Cfg cf, Geo g, Ctl* ctl, P64 P, N64 Nd, Sort S) {
    EP_ACTIVE(ctl);
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nnode) return;
    const int np = P.np;
    int i[3];
    node_coords<D>(n, g, i);
    double xn[3];
#pragma unroll
    for (int d = 0; d < D; ++d) xn[d] = g.ax[d][i[d]];
    const double gz = ctl->g[D - 1];
    const bool tpic = cf.trsfr == EP_TRSFR_TPIC, apic = cf.trsfr == EP_TRSFR_APIC;
    double m = 0.0, pm[3] = {0.0, 0.0, 0.0}, f[3] = {0.0, 0.0, 0.0};
    const int b = S.node_start[n], e = S.node_start[n + 1];
    for (int k = b; k < e; ++k) {
        int p = S.node_list[k];
        int o[3];
        offsets_of<D>(g, i, P.p2e[p], o);
        double N[4];
        shape_at<D>(P, np, p, o, N);
        double Om = P.Om[p];
        double ms = P.rho[p] * Om;
        m = m + N[0] * ms;
        if (D == 2) {
            double sxx = P.sig[0][p], syy = P.sig[1][p], sxy = P.sig[2][p];
            if (apic) {
                // N ms (v + (B D⁻¹) Δnp) (p2n.jl:226)
                const double dl[2] = {xn[0] - P.xo[0][p], xn[1] - P.xo[1][p]};
                double C[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) C[k] = P.BD[k][p];
                pm[0] = pm[0] + N[0] * ms * (P.v[0][p] + apic_row<2>(C, 0, dl));
                pm[1] = pm[1] + N[0] * ms * (P.v[1][p] + apic_row<2>(C, 1, dl));
            } else if (!tpic) {
                double px = ms * P.v[0][p], py = ms * P.v[1][p];
                pm[0] = pm[0] + N[0] * px;
                pm[1] = pm[1] + N[0] * py;
            } else {
                double dx = xn[0] - P.xo[0][p], dy = xn[1] - P.xo[1][p];
                pm[0] = pm[0] + N[0] * ms * (P.v[0][p] + P.dv[0][p] * dx + P.dv[2][p] * dy);
                pm[1] = pm[1] + N[0] * ms * (P.v[1][p] + P.dv[1][p] * dx + P.dv[3][p] * dy);
            }
            f[0] = f[0] + -(Om * (N[1] * sxx + N[2] * sxy));
            f[1] = f[1] + -(Om * (N[1] * sxy + N[2] * syy) - N[0] * (ms * gz));
        } else {
            double sxx = P.sig[0][p], syy = P.sig[1][p], szz = P.sig[2][p];
            double syx = P.sig[5][p], szy = P.sig[3][p], szx = P.sig[4][p];
            if (apic) {
                const double dl[3] = {xn[0] - P.xo[0][p], xn[1] - P.xo[1][p], xn[2] - P.xo[2][p]};
                double C[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) C[k] = P.BD[k][p];
                pm[0] = pm[0] + N[0] * ms * (P.v[0][p] + apic_row<3>(C, 0, dl));
                pm[1] = pm[1] + N[0] * ms * (P.v[1][p] + apic_row<3>(C, 1, dl));
                pm[2] = pm[2] + N[0] * ms * (P.v[2][p] + apic_row<3>(C, 2, dl));
            } else if (!tpic) {
                double px = ms * P.v[0][p], py = ms * P.v[1][p], pz = ms * P.v[2][p];
                pm[0] = pm[0] + N[0] * px;
                pm[1] = pm[1] + N[0] * py;
                pm[2] = pm[2] + N[0] * pz;
            } else {
                double dx = xn[0] - P.xo[0][p], dy = xn[1] - P.xo[1][p], dz = xn[2] - P.xo[2][p];
                pm[0] = pm[0] + N[0] * ms * (P.v[0][p] + P.dv[0][p] * dx + P.dv[3][p] * dy + P.dv[6][p] * dz);
                pm[1] = pm[1] + N[0] * ms * (P.v[1][p] + P.dv[1][p] * dx + P.dv[4][p] * dy + P.dv[7][p] * dz);
                pm[2] = pm[2] + N[0] * ms * (P.v[2][p] + P.dv[2][p] * dx + P.dv[5][p] * dy + P.dv[8][p] * dz);
            }
            f[0] = f[0] + -(Om * (N[1] * sxx + N[2] * syx + N[3] * szx));
            f[1] = f[1] + -(Om * (N[1] * syx + N[2] * syy + N[3] * szy));
            f[2] = f[2] + -(Om * (N[1] * szx + N[2] * szy + N[3] * szz) - N[0] * (ms * gz));
        }
    }
    Nd.m[n] = m;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        Nd.p[d][n] = pm[d];
        Nd.oobf[d][n] = f[d];
    }
}

// Grid momentum update with damping and Dirichlet masks (solve.jl:14-40).
template <int D>
__global__ void k_solve64(Cfg cf, Geo g, Ctl* ctl, N64 Nd) {
    EP_ACTIVE(ctl);
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nnode) return;
    const double dt = ctl->dt, eta = cf.damping;
    double m = Nd.m[n];
    double a[3] = {0.0, 0.0, 0.0}, v[3] = {0.0, 0.0, 0.0};
    if (m != 0.0) {
        double f[3], pm[3];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            f[d] = Nd.oobf[d][n];
            pm[d] = Nd.p[d][n];
        }
        for (int d = 0; d < D; ++d) {
            if (g.bcs[(size_t)d * g.nnode + n]) {
                a[d] = 0.0;
                v[d] = 0.0;
            } else {
                double mi = 1.0 / m;
                double Dm = eta * jnorm<D>(f) * jsign(pm[d] * mi);
                if (fabs(pm[d] * mi) >= 1.0e-3) f[d] = f[d] - Dm;
                a[d] = f[d] * mi;
                v[d] = (pm[d] + dt * f[d]) * mi;
            }
        }
#pragma unroll
        for (int d = 0; d < D; ++d) Nd.oobf[d][n] = f[d];
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
        Nd.a[d][n] = a[d];
        Nd.v[d][n] = v[d];
    }
}

// stencil walk helper: calls fn(slot, node, N[]) for every valid slot in ascending slot order
template <int D, class F>
__device__ __forceinline__ void for_slots(const Geo& g, const P64& P, int np, int p, F fn) {
    int e[3];
    cell_coords<D>(P.p2e[p], g, e);
    const int NN = D == 2 ? 16 : 64;
    for (int s = 0; s < NN; ++s) {
        int o[3], i[3];
        slot_offsets<D>(s, o);
        bool ok = true;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            i[d] = e[d] - 1 + o[d];
            ok = ok && i[d] >= 0 && i[d] < g.nno[d];
        }
        if (!ok) continue;
        double N[4];
        shape_at<D>(P, np, p, o, N);
        fn(s, node_id<D>(i, g), N);
    }
}

// G2P PIC/FLIP blend, position update and vmax (n2p.jl:14-40).
template <int D>
__global__ void k_g2p64(Cfg cf, Geo g, Ctl* ctl, P64 P, N64 Nd) {
    EP_ACTIVE(ctl);
    const int np = P.np;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np || P.p2e[p] < 0) return;
    const double dt = ctl->dt, Cpf = cf.Cpf;
    for (int d = 0; d < D; ++d) {
        double vpic = 0.0, aflip = 0.0;
        for_slots<D>(g, P, np, p, [&](int, int n, const double* N) { vpic = vpic + N[0] * Nd.v[d][n]; });
        for_slots<D>(g, P, np, p, [&](int, int n, const double* N) { aflip = aflip + N[0] * Nd.a[d][n]; });
        double vp = P.v[d][p];
        vp = Cpf * (vp + dt * aflip) + (1.0 - Cpf) * vpic;
        P.v[d][p] = vp;
        P.x[d][p] = P.x[d][p] + dt * vpic;
        atomic_max_abs(&ctl->vmax_bits[d], vp);
    }
    if (cf.trsfr == EP_TRSFR_APIC) {
        // Bij (mapsto/Bij.jl:14-26): Σ N (v_n Δnpᵀ) with the grid velocity of the solve (before the
        // mUSL re-projection, n2p.jl:60-62) and the step-start offsets
        double B[D * D];
#pragma unroll
        for (int k = 0; k < D * D; ++k) B[k] = 0.0;
        for_slots<D>(g, P, np, p, [&](int, int n, const double* N) {
            int ic[3];
            node_coords<D>(n, g, ic);
            double dl[3], vn[3];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                dl[d] = g.ax[d][ic[d]] - P.xo[d][p];
                vn[d] = Nd.v[d][n];
            }
#pragma unroll
            for (int b = 0; b < D; ++b)
#pragma unroll
                for (int a = 0; a < D; ++a) B[a + D * b] = B[a + D * b] + N[0] * (vn[a] * dl[b]);
        });
#pragma unroll
        for (int k = 0; k < D * D; ++k) P.B[k][p] = B[k];
    }
}

// mUSL re-projection: p_n = Σ N (ρΩ) v_p, then v_n = p_n / m_n (augm.jl:13-53).
template <int D>
__global__ void k_augm64(Geo g, Ctl* ctl, P64 P, N64 Nd, Sort S) {
    EP_ACTIVE(ctl);
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nnode) return;
    const int np = P.np;
    int i[3];
    node_coords<D>(n, g, i);
    double pm[3] = {0.0, 0.0, 0.0};
    const int b = S.node_start[n], e = S.node_start[n + 1];
    for (int k = b; k < e; ++k) {
        int p = S.node_list[k];
        int o[3];
        offsets_of<D>(g, i, P.p2e[p], o);
        double N[4];
        shape_at<D>(P, np, p, o, N);
        double mp = P.rho[p] * P.Om[p];
#pragma unroll
        for (int d = 0; d < D; ++d) pm[d] = pm[d] + N[0] * (mp * P.v[d][p]);
    }
    double m = Nd.m[n];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        Nd.p[d][n] = pm[d];
        double v = 0.0;
        if (m != 0.0) v = g.bcs[(size_t)d * g.nnode + n] ? 0.0 : pm[d] * (1.0 / m);
        Nd.v[d][n] = v;
    }
}

// Velocity gradient, deformation, volume and GIMP domain (deform.jl, domain.jl).
template <int D>
__global__ void k_deform64(Cfg cf, Geo g, Ctl* ctl, P64 P, N64 Nd) {
    EP_ACTIVE(ctl);
    const int np = P.np;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np || P.p2e[p] < 0) return;
    const double dt = ctl->dt;
    double gv[D * D];
#pragma unroll
    for (int k = 0; k < D * D; ++k) gv[k] = 0.0;
    for_slots<D>(g, P, np, p, [&](int, int n, const double* N) {
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
            for (int b = 0; b < D; ++b) gv[a + D * b] = gv[a + D * b] + N[b + 1] * Nd.v[a][n];
    });
    double dF[D * D], F[D * D], Fn[D * D];
#pragma unroll
    for (int b = 0; b < D; ++b)
#pragma unroll
        for (int a = 0; a < D; ++a) {
            dF[a + D * b] = (a == b ? 1.0 : 0.0) + dt * gv[a + D * b];
            F[a + D * b] = P.F[a + D * b][p];
        }
    matmul<D>(dF, F, Fn);
    double dJ = det_lu<D>(dF);
    double J = det_lu<D>(Fn);
    double Om = J * P.Om0[p];
    P.dJ[p] = dJ;
    P.J[p] = J;
    P.Om[p] = Om;
    if (cf.deform == EP_DEFORM_FINITE) {
        P.rho[p] = P.rho0[p] / J;
        P.n[p] = 1.0 - 1.0 / J * (1.0 - P.n0[p]);
    }
#pragma unroll
    for (int k = 0; k < D * D; ++k) {
        P.dv[k][p] = gv[k];
        P.dF[k][p] = dF[k];
        P.F[k][p] = Fn[k];
    }
    if (cf.basis == EP_BASIS_GIMPM) {
        double lp[3], l0[3];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            lp[d] = P.l[d][p];
            l0[d] = P.l0[d][p];
        }
        switch (cf.how) {
            case EP_HOW_UNDEFORMED:
                for (int d = 0; d < D; ++d) lp[d] = l0[d];
                break;
            case EP_HOW_DETFIJ: {
                double j = det_lu<D>(Fn);
                for (int d = 0; d < D; ++d) lp[d] = l0[d] * j;
            } break;
            case EP_HOW_DETDFIJ: {
                double j = det_lu<D>(dF);
                for (int d = 0; d < D; ++d) lp[d] = lp[d] * j;
            } break;
            case EP_HOW_FII:
                for (int d = 0; d < D; ++d) lp[d] = l0[d] * Fn[d + D * d];
                break;
            case EP_HOW_DFII:
                for (int d = 0; d < D; ++d) lp[d] = lp[d] * dF[d + D * d];
                break;
            case EP_HOW_UII:
            case EP_HOW_DUII: {
                const double* A = (cf.how == EP_HOW_UII) ? Fn : dF;
                double C[D * D], lam[D], V[D * D], s[D], U[D * D];
                matmul_at<D>(A, A, C);
                eig_sym<D>(C, lam, V);
                for (int d = 0; d < D; ++d) s[d] = sqrt(lam[d]);
                vdvt<D>(V, s, U);
                if (cf.how == EP_HOW_UII)
                    for (int d = 0; d < D; ++d) lp[d] = U[d + D * d] * l0[d];
                else
                    for (int d = 0; d < D; ++d) lp[d] = U[d + D * d] * lp[d];
            } break;
            default:
                break;
        }
#pragma unroll
        for (int d = 0; d < D; ++d) P.l[d][p] = lp[d];
    }
}

// F-bar: ΔJ_n = Σ N (ρΩ) ΔJ_p / m_n (volumetric.jl:1-22).
template <int D>
__global__ void k_dJ64(Geo g, Ctl* ctl, P64 P, N64 Nd, Sort S) {
    EP_ACTIVE(ctl);
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nnode) return;
    const int np = P.np;
    int i[3];
    node_coords<D>(n, g, i);
    double s = 0.0;
    const int b = S.node_start[n], e = S.node_start[n + 1];
    for (int k = b; k < e; ++k) {
        int p = S.node_list[k];
        int o[3];
        offsets_of<D>(g, i, P.p2e[p], o);
        double N[4];
        shape_at<D>(P, np, p, o, N);
        s = s + N[0] * ((P.rho[p] * P.Om[p]) * P.dJ[p]);
    }
    double m = Nd.m[n];
    Nd.dJ[n] = (m == 0.0) ? 0.0 : s / m;
}

template <int D>
__device__ __forceinline__ void retmap_point(const Cfg& cf, const Mat& mt, Ctl* ctl, const P64& P, int p) {
    const int NS = D == 2 ? 3 : 6;
    const bool fin = cf.deform == EP_DEFORM_FINITE;
    double s[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) s[k] = fin ? P.tau[k][p] : P.sig[k][p];
    double ep1 = P.ep1[p], ep2 = P.ep2[p];
    bool write = false, rebuild = false;
    double dl = P.dlam[p];
    if (cf.cons == EP_CONS_DP) {
        dl = (D == 2) ? dp_return<3>(s, ep2, P.c0[p], P.cr[p], P.tphi[p], 0.0, 0.0, mt.Hp, mt.Kc, mt.Gc, &ep1)
                      : dp_return<6>(s, ep2, P.c0[p], P.cr[p], 0.0, P.sphi[p], P.cphi[p], mt.Hp, mt.Kc, mt.Gc, &ep1);
        P.dlam[p] = dl;
        write = true;
        rebuild = fin;
    } else if (cf.cons == EP_CONS_J2) {
        int y = j2_return<NS>(s, ep2, P.c0[p], P.cr[p], mt.Hp, mt.Del, &ep1);
        write = y != 0;
        rebuild = fin && y;
    } else {
        // MC (2d, MCRetMap.jl) or modified Cam-Clay (camCmodRetMap.jl): ϵ = tensor(Del \ σ, ½) of the
        // returned stress in both frameworks, b_e = exp(2ϵ) in finite strain
        int y;
        if (cf.cons == EP_CONS_MC) {
            y = mc_return(s, ep2, P.c0[p], P.cr[p], P.sphi[p], P.cphi[p], mt.Hp, mt.Del, mt.DelLU, mt.piv, &ep1);
            if (y < 0) set_err(ctl, EP_ERR_NONCONVERGED, p);
        } else {
            double ev = P.epv[p];
            y = camc_return<NS>(s, ep2, &ev, mt.Kc, mt.Del, &ep1);
            if (y > 0) P.epv[p] = ev;
        }
        write = y > 0;
        rebuild = fin && y > 0;
        if (y > 0 && !fin) {
            double eps[D * D];
            strain_from_stress<D>(s, mt.DelLU, mt.piv, eps);
#pragma unroll
            for (int k = 0; k < D * D; ++k) P.eps[k][p] = eps[k];
        }
    }
    if (write) {
        P.ep1[p] = ep1;
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            if (fin) P.tau[k][p] = s[k];
            else P.sig[k][p] = s[k];
        }
    }
    if (rebuild) {
        double eps[D * D], b[D * D];
        finite_rebuild_b<D>(s, mt.DelLU, mt.piv, eps, b);
#pragma unroll
        for (int k = 0; k < D * D; ++k) {
            P.eps[k][p] = eps[k];
            P.b[k][p] = b[k];
        }
    }
    unsigned mask = __activemask();
    unsigned bal = __ballot_sync(mask, P.dlam[p] != 0.0);
    if ((threadIdx.x & 31) == __ffs(mask) - 1) atomicAdd((unsigned long long*)&ctl->plastic, (unsigned long long)__popc(bal));
}

template <int D>
__device__ __forceinline__ void check_finite(Ctl* ctl, const P64& P, int p, bool fin) {
    const int NS = D == 2 ? 3 : 6;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < D; ++d) ok = ok && isfinite(P.x[d][p]) && isfinite(P.v[d][p]);
#pragma unroll
    for (int k = 0; k < NS; ++k) ok = ok && isfinite(fin ? P.tau[k][p] : P.sig[k][p]);
    if (!ok) set_err(ctl, EP_ERR_NONFINITE, p);
}

// ΔJp scaling of ΔF, elastic predictor and, without nonlocal averaging, the return map.
template <int D>
__global__ void k_elast64(Cfg cf, Geo g, Mat mt, Ctl* ctl, P64 P, N64 Nd, int plastic_phase) {
    EP_ACTIVE(ctl);
    const int np = P.np;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np || P.p2e[p] < 0) return;
    double dF[D * D];
#pragma unroll
    for (int k = 0; k < D * D; ++k) dF[k] = P.dF[k][p];
    if (cf.locking) {
        double s = 0.0;
        const double dJp = P.dJ[p];
        for_slots<D>(g, P, np, p, [&](int, int n, const double* N) { s = s + N[0] * Nd.dJ[n] / dJp; });
        double f = (D == 2) ? sqrt(s) : ep_pow(s, 1.0 / 3.0);
#pragma unroll
        for (int k = 0; k < D * D; ++k) {
            dF[k] = dF[k] * f;
            P.dF[k][p] = dF[k];
        }
    }
    const int NS = D == 2 ? 3 : 6;
    const bool fin = cf.deform == EP_DEFORM_FINITE;
    if (fin) {
        double b[D * D], eps[D * D], tau[NS];
#pragma unroll
        for (int k = 0; k < D * D; ++k) b[k] = P.b[k][p];
        finite_elast<D>(dF, b, eps, tau, mt.Del);
#pragma unroll
        for (int k = 0; k < D * D; ++k) {
            P.b[k][p] = b[k];
            P.eps[k][p] = eps[k];
        }
#pragma unroll
        for (int k = 0; k < NS; ++k) P.tau[k][p] = tau[k];
    } else {
        double sig[NS], eps[D * D], w[D * D], sJ[D * D];
#pragma unroll
        for (int k = 0; k < NS; ++k) sig[k] = P.sig[k][p];
        infinitesimal_elast<D>(dF, sig, eps, w, sJ, mt.Del, cf.jaumann);
#pragma unroll
        for (int k = 0; k < NS; ++k) P.sig[k][p] = sig[k];
#pragma unroll
        for (int k = 0; k < D * D; ++k) {
            P.eps[k][p] = eps[k];
            P.w[k][p] = w[k];
            P.sJ[k][p] = sJ[k];
        }
    }
    if (plastic_phase && !cf.nonloc) {
        P.ep2[p] = P.ep1[p];
        retmap_point<D>(cf, mt, ctl, P, p);
    }
    if (!(plastic_phase && cf.nonloc)) check_finite<D>(ctl, P, p, fin);
}

// ---------------------------------------------------------------------------
// Nonlocal averaging of ϵpII in the reference's serial visiting order
// (nonlocal.jl:18-47 with plast.jl:51-59), one warp per point.  For a point p
// that yielded in the previous return (Δλ != 0), with N(p) the points of the
// cells within ±ceil(ls/h) of p's cell (p included), the serial sweep gives
//   W[p]  = Σ_{r in N(p), r plastic, r<p} ω(r,p)   (added while r is visited)
//         + Σ_{q in N(p), not (q plastic and q<p)} ω(p,q)   (p's own visit)
//   ϵ2[p] = Σ_{q in N(p), not (q plastic and q<p)} (ω(p,q)/W[p]) ϵ1[q]
// each sum in ascending id order; ϵ2[p] = ϵ1[p] when W[p] <= 1e-16 and 0 for
// non-plastic points.  ω = (d/ls) exp(-(d/ls)^2) with d the distance in the
// first two coordinates (nonlocal.jl:27-28).
// ---------------------------------------------------------------------------
constexpr int NL_CAP = 2048;

template <int D>
__global__ void __launch_bounds__(32) k_nonlocal64(Cfg cf, Geo g, Ctl* ctl, P64 P, Sort S) {
    EP_ACTIVE(ctl);
    __shared__ int qs[NL_CAP];
    __shared__ double om[NL_CAP];
    const int p = blockIdx.x;
    const int lane = threadIdx.x;
    if (p >= P.np) return;
    if (P.dlam[p] == 0.0 || P.p2e[p] < 0) {
        if (lane == 0) P.ep2[p] = 0.0;
        return;
    }
    int e[3];
    cell_coords<D>(P.p2e[p], g, e);
    int lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        lo[d] = max(e[d] - g.nnel[d], 0);
        hi[d] = min(e[d] + g.nnel[d], g.nel[d] - 1);
    }
    // gather the candidate ids (cell order), count them
    int L = 0;
    auto visit_cells = [&](auto fn) {
        if (D == 2) {
            for (int a = lo[0]; a <= hi[0]; ++a)
                for (int b = lo[1]; b <= hi[1]; ++b) fn(b + g.nel[1] * a);
        } else {
            for (int k = lo[1]; k <= hi[1]; ++k)
                for (int a = lo[0]; a <= hi[0]; ++a)
                    for (int b = lo[2]; b <= hi[2]; ++b) fn(b + g.nel[2] * a + g.nel[2] * g.nel[0] * k);
        }
    };
    visit_cells([&](int c) { L += S.cell_start[c + 1] - S.cell_start[c]; });
    const double ls = cf.ls;
    const double xp0 = P.x[0][p], xp1 = P.x[1][p];
    if (L <= NL_CAP) {
        int pos = 0;
        visit_cells([&](int c) {
            int b = S.cell_start[c], n = S.cell_start[c + 1] - b;
            for (int k = lane; k < n; k += 32) qs[pos + k] = S.cell_list[b + k];
            pos += n;
        });
        int P2 = 32;
        while (P2 < L) P2 <<= 1;
        for (int k = L + lane; k < P2; k += 32) qs[k] = INT_MAX;
        __syncwarp();
        for (int k = 2; k <= P2; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int t = lane; t < P2; t += 32) {
                    int q = t ^ j;
                    if (q > t) {
                        int a = qs[t], c = qs[q];
                        bool asc = (t & k) == 0;
                        if ((a > c) == asc) { qs[t] = c; qs[q] = a; }
                    }
                }
                __syncwarp();
            }
        for (int t = lane; t < L; t += 32) {
            int q = qs[t];
            double xi = xp0 - P.x[0][q], et = xp1 - P.x[1][q];
            double dd = sqrt(xi * xi + et * et);
            double r = dd / ls;
            om[t] = dd / ls * ep_exp(-(r * r));
        }
        __syncwarp();
        if (lane == 0) {
            double W = 0.0;
            for (int t = 0; t < L; ++t) {
                int q = qs[t];
                if (q >= p) break;
                if (P.dlam[q] != 0.0) W = W + om[t];
            }
            for (int t = 0; t < L; ++t) {
                int q = qs[t];
                if (q < p && P.dlam[q] != 0.0) continue;
                W = W + om[t];
            }
            double s = 0.0;
            if (!(W > 1e-16)) {
                s = P.ep1[p];
            } else {
                for (int t = 0; t < L; ++t) {
                    int q = qs[t];
                    if (q < p && P.dlam[q] != 0.0) continue;
                    s = s + (om[t] / W) * P.ep1[q];
                }
            }
            P.ep2[p] = s;
        }
        return;
    }
    // rare: more candidates than the shared buffer holds -> walk them in
    // ascending order by repeated minimum selection (slow, still exact)
    if (lane != 0) return;
    double W = 0.0;
    for (int pass = 0; pass < 3; ++pass) {
        double s = 0.0;
        int last = -1;
        if (pass == 2 && !(W > 1e-16)) {
            P.ep2[p] = P.ep1[p];
            return;
        }
        while (true) {
            int best = INT_MAX;
            visit_cells([&](int c) {
                for (int k = S.cell_start[c]; k < S.cell_start[c + 1]; ++k) {
                    int q = S.cell_list[k];
                    if (q > last && q < best) best = q;
                }
            });
            if (best == INT_MAX) break;
            last = best;
            int q = best;
            bool plq = P.dlam[q] != 0.0;
            if (pass == 0 && !(q < p && plq)) continue;
            if (pass >= 1 && (q < p && plq)) continue;
            double xi = xp0 - P.x[0][q], et = xp1 - P.x[1][q];
            double dd = sqrt(xi * xi + et * et);
            double r = dd / ls;
            double w = dd / ls * ep_exp(-(r * r));
            if (pass < 2) W = W + w;
            else s = s + (w / W) * P.ep1[q];
        }
        if (pass == 2) P.ep2[p] = s;
    }
}

template <int D>
__global__ void k_retmap64(Cfg cf, Mat mt, Ctl* ctl, P64 P) {
    EP_ACTIVE(ctl);
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.np || P.p2e[p] < 0) return;
    retmap_point<D>(cf, mt, ctl, P, p);
    check_finite<D>(ctl, P, p, cf.deform == EP_DEFORM_FINITE);
}

// ---------------------------------------------------------------------------
// control block
__global__ void k_ctl_begin_run(Ctl* c, int dim, double h0, double h1, double h2, double cw) {
    ctl_begin_run(c, dim, h0, h1, h2, cw);
}

__global__ void k_ctl_begin_step(Ctl* c) {
    c->active = c->err ? 0 : 1;
    for (int i = 0; i < 3; ++i) c->vmax_bits[i] = 0ull;
    c->plastic = 0;
}

__global__ void k_ctl_end(Ctl* c) { ctl_end(c); }

void launch_ctl_begin_run(Ctl* ctl, const Geo& g, double c, cudaStream_t s) {
    k_ctl_begin_run<<<1, 1, 0, s>>>(ctl, g.dim, g.h[0], g.h[1], g.h[2], c);
}
void launch_ctl_begin_step(Ctl* ctl, int, cudaStream_t s) { k_ctl_begin_step<<<1, 1, 0, s>>>(ctl); }

// the caller's dt, g and phase of one step into the control block (its other fields stay the device's)
__global__ void k_ctl_set_step(Ctl* c, double dt, double g0, double g1, double g2, int phase) {
    c->dt = dt;
    c->g[0] = g0;
    c->g[1] = g1;
    c->g[2] = g2;
    c->phase = phase;
}
void launch_ctl_set_step(Ctl* ctl, double dt, const double* g, int phase, cudaStream_t s) {
    k_ctl_set_step<<<1, 1, 0, s>>>(ctl, dt, g[0], g[1], g[2], phase);
}
void launch_ctl_end(Ctl* ctl, cudaStream_t s) { k_ctl_end<<<1, 1, 0, s>>>(ctl); }

// ---------------------------------------------------------------------------
template <int D, int BASIS>
static void step_impl(const Fp64Ctx& c, int phase, cudaStream_t s) {
    const int np = c.np, nnode = c.g.nnode, ncell = c.g.ncell;
    const int TB = 128;
    const int gp = (np + TB - 1) / TB, gn = (nnode + TB - 1) / TB;
    long long L = 0;
    Prof* pr = (c.prof && c.prof->on) ? c.prof : nullptr;
    auto mark = [&](const char* nm) {
        if (pr) pr->mark(nm, s);
    };
    cudaMemsetAsync(c.S.cell_count, 0, sizeof(int) * ncell, s);
    cudaMemsetAsync(c.S.node_cursor, 0, sizeof(int) * nnode, s);
    mark("memset");
    const bool nl = phase == EP_PHASE_ELASTOPLASTIC && c.cf.nonloc;
    if (np > 0) { k_bin64<D, BASIS><<<gp, TB, 0, s>>>(c.cf, c.g, c.ctl, c.P, c.S.cell_count); ++L; mark("bin64"); }
    if (nl) {
        cudaMemsetAsync(c.S.cell_cursor, 0, sizeof(int) * ncell, s);
        launch_exclusive_scan(c.S.cell_count, c.S.cell_start, ncell, c.S.scan_tmp, s);
        launch_place_cells(c.P.p2e, np, c.S.cell_start, c.S.cell_cursor, c.S.cell_list, c.ctl, s);
        launch_segsort(c.S.cell_start, ncell, c.S.cell_list, s);
        L += 5;
        mark("cell_lists");
    }
    k_count_nodes<D><<<gn, TB, 0, s>>>(c.g, c.ctl, c.S.cell_count, c.S.node_count);
    launch_exclusive_scan(c.S.node_count, c.S.node_start, nnode, c.S.scan_tmp, s);
    if (np > 0) k_place_nodes<D><<<gp, TB, 0, s>>>(c.g, c.ctl, c.P.p2e, np, c.S.node_start, c.S.node_cursor, c.S.node_list);
    mark("node_lists");
    launch_segsort(c.S.node_start, nnode, c.S.node_list, s);
    mark("segsort_nodes");
    L += 6;
    k_p2g64<D><<<gn, TB, 0, s>>>(c.cf, c.g, c.ctl, c.P, c.N, c.S);
    mark("p2g64");
    k_solve64<D><<<gn, TB, 0, s>>>(c.cf, c.g, c.ctl, c.N);
    mark("solve64");
    L += 2;
    if (np > 0) { k_g2p64<D><<<gp, TB, 0, s>>>(c.cf, c.g, c.ctl, c.P, c.N); ++L; mark("g2p64"); }
    if (c.cf.musl) { k_augm64<D><<<gn, TB, 0, s>>>(c.g, c.ctl, c.P, c.N, c.S); ++L; mark("augm64"); }
    if (np > 0) { k_deform64<D><<<gp, TB, 0, s>>>(c.cf, c.g, c.ctl, c.P, c.N); ++L; mark("deform64"); }
    if (c.cf.locking) { k_dJ64<D><<<gn, TB, 0, s>>>(c.g, c.ctl, c.P, c.N, c.S); ++L; mark("dJ64"); }
    if (np > 0) {
        k_elast64<D><<<gp, TB, 0, s>>>(c.cf, c.g, c.mt, c.ctl, c.P, c.N, phase == EP_PHASE_ELASTOPLASTIC);
        ++L;
        mark("elast64");
        if (nl) {
            k_nonlocal64<D><<<np, 32, 0, s>>>(c.cf, c.g, c.ctl, c.P, c.S);
            mark("nonlocal64");
            k_retmap64<D><<<gp, TB, 0, s>>>(c.cf, c.mt, c.ctl, c.P);
            mark("retmap64");
            L += 2;
        }
    }
    if (c.launches) *c.launches += L;
}

void fp64_step(const Fp64Ctx& c, int phase, cudaStream_t s) {
    if (c.cf.dim == 2) {
        if (c.cf.basis == EP_BASIS_BSMPM) step_impl<2, EP_BASIS_BSMPM>(c, phase, s);
        else if (c.cf.basis == EP_BASIS_GIMPM) step_impl<2, EP_BASIS_GIMPM>(c, phase, s);
        else step_impl<2, EP_BASIS_SMPM>(c, phase, s);
    } else {
        if (c.cf.basis == EP_BASIS_BSMPM) step_impl<3, EP_BASIS_BSMPM>(c, phase, s);
        else if (c.cf.basis == EP_BASIS_GIMPM) step_impl<3, EP_BASIS_GIMPM>(c, phase, s);
        else step_impl<3, EP_BASIS_SMPM>(c, phase, s);
    }
}

}  // namespace ep
