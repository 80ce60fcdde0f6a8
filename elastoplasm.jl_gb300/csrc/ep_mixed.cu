// ep_mixed.cu -- the mixed-precision MPM step (2d), the fast path.
//
// Same method and call order as the reference step (worflow.jl:80-82), with
// transfers and grid arithmetic in FP32 and FP64 where accumulation or
// cancellation needs it:
//   * positions, F and b_e are FP64 state; their per-step increments are
//     formed in FP32 (they are small: dt∇v ~ 1e-4) and added in FP64;
//   * F-bar carries δJ = ΔJ - 1 instead of ΔJ, so no FP32 cancellation
//     against 1 happens (volumetric.jl:1-36 in "increment" form);
//   * log b_e and exp(2ε) of the finite-strain predictor/return
//     (elast.jl:49-54, DP.jl:63-66) use the closed spectral form of a
//     symmetric 2x2 tensor A = m I + A_d (A_d deviatoric, eigenvalues m ± r):
//       log A = (log m + ½ log(1 - x²)) I + (atanh(x)/x)/m · A_d,  x = r/m,
//       exp(2E) = e^{2 e_m} (cosh(2s) I + sinh(2s)/s · E_d),       s² = ½ tr(E_d²),
//     with log m and e^{2 e_m} (the isotropic part, which carries the
//     magnitude) in FP64 and the deviatoric factors in FP32 (arguments x², s²
//     are small invariants).  No explicit eigenvectors are needed.
//   * the accumulated plastic strain is FP64.
//
// Transfers are cell-centric: one thread per cell walks the points of its
// cell (cell lists from a counting sort, rebuilt every step) and accumulates
// its 16 stencil nodes' sums in registers, then adds them to the grid with
// FP32 atomics -- one atomic per node and quantity per cell instead of per
// point.  Kernels of one step:
//   km_p2g    P2G of m, p, f                      (p2n.jl:135-155)      cell
//   km_solve  grid update                         (solve.jl:14-40)      node
//   km_g2p    PIC/FLIP, positions, vmax, mUSL P2G, next cell counts
//             (n2p.jl:14-40, augm.jl:13-25, tplgy.jl:43-62)             cell
//   km_vmusl  mUSL nodal velocity                 (augm.jl:37-53)       node
//   scan of the next cell counts
//   km_fbar   ∇v, δJ and its P2G; next cell lists (deform.jl, volumetric.jl:1-11) cell
//   km_dJn    nodal δJ                            (volumetric.jl:12-22) node
//   km_cons   F-bar, F, elastic predictor, DP/J2  (volumetric.jl:23-36, deform.jl,
//             elast.jl, DP.jl, J2.jl)                                   cell
#include <climits>

#include "../../include/epgpu.h"
#include "ep_internal.h"
#include "ep_mixed.cuh"

namespace ep {

#define EP_ACTIVE(ctl) \
    if (!(ctl)->active) return

// ---------------------------------------------------------------------------
// FP32 shape pieces (the polynomials of bsmpm.jl:1-62, gimpm.jl:1-14, smpm.jl:1-10)
__device__ __forceinline__ void bs32(int cls, float x, float& f, float& df) {
    float F = 0.f, G = 0.f;
    const float x2 = x * x, x3 = x2 * x;
    if (cls == BS_T3) {
        if (-2.f <= x && x <= -1.f) { F = (1.f / 6.f) * x3 + x2 + 2.f * x + (4.f / 3.f); G = 0.5f * x2 + 2.f * x + 2.f; }
        else if (-1.f <= x && x <= 0.f) { F = -0.5f * x3 - x2 + (2.f / 3.f); G = -1.5f * x2 - 2.f * x; }
        else if (0.f <= x && x <= 1.f) { F = 0.5f * x3 - x2 + (2.f / 3.f); G = 1.5f * x2 - 2.f * x; }
        else if (1.f <= x && x <= 2.f) { F = (-1.f / 6.f) * x3 + x2 - 2.f * x + (4.f / 3.f); G = -0.5f * x2 + 2.f * x - 2.f; }
    } else if (cls == BS_T1) {
        if (-2.f <= x && x <= -1.f) { F = (1.f / 6.f) * x3 + x2 + 2.f * x + (4.f / 3.f); G = 0.5f * x2 + 2.f * x + 2.f; }
        else if (-1.f <= x && x <= 0.f) { F = (-1.f / 6.f) * x3 + x + 1.f; G = -0.5f * x2 + 1.f; }
        else if (0.f <= x && x <= 1.f) { F = (1.f / 6.f) * x3 - x + 1.f; G = 0.5f * x2 - 1.f; }
        else if (1.f <= x && x <= 2.f) { F = (-1.f / 6.f) * x3 + x2 - 2.f * x + (4.f / 3.f); G = -0.5f * x2 + 2.f * x - 2.f; }
    } else if (cls == BS_T2) {
        if (-1.f <= x && x <= 0.f) { F = (-1.f / 3.f) * x3 - x2 + (2.f / 3.f); G = -1.f * x2 - 2.f * x; }
        else if (0.f <= x && x <= 1.f) { F = 0.5f * x3 - x2 + (2.f / 3.f); G = 1.5f * x2 - 2.f * x; }
        else if (1.f <= x && x <= 2.f) { F = (-1.f / 6.f) * x3 + x2 - 2.f * x + (4.f / 3.f); G = -0.5f * x2 + 2.f * x - 2.f; }
    } else if (cls == BS_T4) {
        if (-2.f <= x && x <= -1.f) { F = (1.f / 6.f) * x3 + x2 + 2.f * x + (4.f / 3.f); G = 0.5f * x2 + 2.f * x + 2.f; }
        else if (-1.f <= x && x <= 0.f) { F = -0.5f * x3 - x2 + (2.f / 3.f); G = -1.5f * x2 - 2.f * x; }
        else if (0.f <= x && x <= 1.f) { F = (1.f / 3.f) * x3 - x2 + (2.f / 3.f); G = x2 - 2.f * x; }
    }
    f = F;
    df = G;
}

__device__ __forceinline__ void gimp32(float d, float h, float lp, float& f, float& df) {
    float S = 0.f, G = 0.f;
    const float a = fabsf(d);
    if (a < lp) {
        S = 1.f - (4.f * d * d + (2.f * lp) * (2.f * lp)) / (8.f * h * lp);
        G = -(8.f * d) / (8.f * h * lp);
    } else if (a <= h - lp) {
        S = 1.f - a / h;
        G = (d > 0.f ? -1.f : (d < 0.f ? 1.f : 0.f)) / h;
    } else if (a < h + lp) {
        const float r = h + lp - a;
        S = r * r / (4.f * h * lp);
        G = -(d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f)) * r / (2.f * h * lp);
    }
    f = S;
    df = G;
}

__device__ __forceinline__ void hat32(float d, float h, float& f, float& df) {
    if (-h < d && d <= 0.f) { f = 1.f + d / h; df = 1.f / h; }
    else if (0.f < d && d <= h) { f = 1.f - d / h; df = -1.f / h; }
    else { f = 0.f; df = 0.f; }
}

// Per-cell stencil description along one direction: node index base (e-1),
// validity of the 4 nodes and their B-spline classes.
struct Axis4 {
    int base;
    signed char cls[4];     // -1: node outside the grid
};

__device__ __forceinline__ Axis4 axis4(const Geo& g, int d, int e) {
    Axis4 a;
    a.base = e - 1;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int i = e - 1 + k;
        a.cls[k] = (i >= 0 && i < g.nno[d]) ? g.cls[d][i] : (signed char)-1;
    }
    return a;
}

// weights and gradients of the 4 nodes along one direction for a point at
// offset dloc = x - x_e (x_e: node e, the left node of the point's cell)
template <int BASIS>
__device__ __forceinline__ void axis_w(const Axis4& a, float dloc, float h, float ih, float lp, float* w, float* dw,
                                       bool& bad) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float f = 0.f, df = 0.f;
        if (a.cls[k] >= 0) {
            const float dk = dloc + h * (float)(1 - k);        // x - x_{e-1+k}
            if (BASIS == EP_BASIS_BSMPM) {
                if (a.cls[k] == BS_INVALID) bad = true;
                bs32(a.cls[k], dk * ih, f, df);
                df *= ih;
            } else if (BASIS == EP_BASIS_GIMPM) {
                gimp32(dk, h, lp, f, df);
            } else {
                hat32(dk, h, f, df);
            }
        }
        w[k] = f;
        dw[k] = df;
    }
}

struct MCtx {
    Cfg cf;
    Geo g;
    Ctl* ctl;
    PM P;
    NM N;
    SM S;
    float Del[9];       // FP32 copy of the 3x3 stiffness (2d)
    float Cmp[9];       // its inverse (compliance), FP32
    float Kc, Gc, Hp;
    double c;           // wave speed
};

// shape function weights of point p in cell (ex, ez), parity buffer cur
template <int BASIS>
__device__ __forceinline__ void point_w2(const MCtx& A, const Axis4& ax, const Axis4& az, int p, int cur, double axe,
                                         double aze, float* wx, float* dwx, float* wz, float* dwz, bool& bad) {
    const float hx = (float)A.g.h[0], hz = (float)A.g.h[1];
    const float dx = (float)(A.P.x[cur][0][p] - axe);
    const float dz = (float)(A.P.x[cur][1][p] - aze);
    const float lx = BASIS == EP_BASIS_GIMPM ? A.P.l[0][p] : 0.f;
    const float lz = BASIS == EP_BASIS_GIMPM ? A.P.l[1][p] : 0.f;
    axis_w<BASIS>(ax, dx, hx, 1.f / hx, lx, wx, dwx, bad);
    axis_w<BASIS>(az, dz, hz, 1.f / hz, lz, wz, dwz, bad);
}

__device__ __forceinline__ int node2(const Geo& g, const Axis4& ax, const Axis4& az, int i, int j) {
    return (az.base + j) + g.nno[1] * (ax.base + i);
}

// ---------------------------------------------------------------------------
// km_p2g: m, p, f of the 16 stencil nodes of a cell, summed over its points
template <int BASIS>
__global__ void __launch_bounds__(128) km_p2g(MCtx A) {
    EP_ACTIVE(A.ctl);
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.g.ncell) return;
    const int cur = A.ctl->parity;
    const int b = A.S.start[cur][c], e = A.S.start[cur][c + 1];
    if (b == e) return;
    const int ex = c / A.g.nel[1], ez = c - ex * A.g.nel[1];
    const Axis4 ax = axis4(A.g, 0, ex), az = axis4(A.g, 1, ez);
    const double axe = A.g.ax[0][ex], aze = A.g.ax[1][ez];
    const float gz = (float)A.ctl->g[1];
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    const bool tpic = A.cf.trsfr == EP_TRSFR_TPIC;
    float am[16], apx[16], apz[16], afx[16], afz[16];
#pragma unroll
    for (int s = 0; s < 16; ++s) am[s] = apx[s] = apz[s] = afx[s] = afz[s] = 0.f;
    bool bad = false;
    const int* list = A.S.list[cur];
    for (int k = b; k < e; ++k) {
        const int p = list[k];
        float wx[4], dwx[4], wz[4], dwz[4];
        point_w2<BASIS>(A, ax, az, p, cur, axe, aze, wx, dwx, wz, dwz, bad);
        const float ms = A.P.mp[p];
        const float vx = A.P.v[0][p], vz = A.P.v[1][p];
        // Ω σ: finite Ω τ / J = Ω0 τ; infinitesimal Ω σ
        const float sc = fin ? A.P.Om0[p] : A.P.Om[p];
        const float txx = sc * A.P.tau[0][p], tzz = sc * A.P.tau[1][p], txz = sc * A.P.tau[2][p];
        float gxx = 0.f, gxz = 0.f, gzx = 0.f, gzz = 0.f, xo = 0.f, zo = 0.f;
        if (tpic) {
            gxx = A.P.dv[0][p]; gzx = A.P.dv[1][p]; gxz = A.P.dv[2][p]; gzz = A.P.dv[3][p];
            xo = (float)(A.P.x[cur][0][p] - axe);
            zo = (float)(A.P.x[cur][1][p] - aze);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int s = j + 4 * i;
                const float N = wx[i] * wz[j], Nx = dwx[i] * wz[j], Nz = wx[i] * dwz[j];
                const float Nm = N * ms;
                am[s] += Nm;
                if (!tpic) {
                    apx[s] += Nm * vx;
                    apz[s] += Nm * vz;
                } else {
                    // δ = x_n - x_p for node (e-1+i, e-1+j)
                    const float dx = (float)(i - 1) * (float)A.g.h[0] - xo;
                    const float dz = (float)(j - 1) * (float)A.g.h[1] - zo;
                    apx[s] += Nm * (vx + gxx * dx + gxz * dz);
                    apz[s] += Nm * (vz + gzx * dx + gzz * dz);
                }
                afx[s] -= Nx * txx + Nz * txz;
                afz[s] -= (Nx * txz + Nz * tzz) - Nm * gz;
            }
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, c);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (ax.cls[i] < 0 || az.cls[j] < 0) continue;
            const int s = j + 4 * i, n = node2(A.g, ax, az, i, j);
            atomicAdd(&A.N.m[n], am[s]);
            atomicAdd(&A.N.p[0][n], apx[s]);
            atomicAdd(&A.N.p[1][n], apz[s]);
            atomicAdd(&A.N.f[0][n], afx[s]);
            atomicAdd(&A.N.f[1][n], afz[s]);
        }
}

// km_solve: grid momentum update with damping and Dirichlet masks (solve.jl:14-40)
__global__ void km_solve(MCtx A) {
    EP_ACTIVE(A.ctl);
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= A.g.nnode) return;
    const float dt = (float)A.ctl->dt, eta = (float)A.cf.damping;
    const float m = A.N.m[n];
    float a[2] = {0.f, 0.f}, v[2] = {0.f, 0.f};
    if (m != 0.f) {
        float f[2] = {A.N.f[0][n], A.N.f[1][n]};
        const float pm[2] = {A.N.p[0][n], A.N.p[1][n]};
        const float mi = 1.f / m;
#pragma unroll
        for (int d = 0; d < 2; ++d) {
            if (A.g.bcs[(size_t)d * A.g.nnode + n]) continue;
            const float nrm = sqrtf(f[0] * f[0] + f[1] * f[1]);
            const float pv = pm[d] * mi;
            const float sg = pv > 0.f ? 1.f : (pv < 0.f ? -1.f : 0.f);
            if (fabsf(pv) >= 1.0e-3f) f[d] -= eta * nrm * sg;
            a[d] = f[d] * mi;
            v[d] = (pm[d] + dt * f[d]) * mi;
        }
        A.N.f[0][n] = f[0];
        A.N.f[1][n] = f[1];
    }
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        A.N.a[d][n] = a[d];
        A.N.v[d][n] = v[d];
        A.N.pm[d][n] = 0.f;
    }
    A.N.dJacc[n] = 0.f;
}

// km_g2p: PIC/FLIP update, new positions, vmax, mUSL momentum P2G, next-cell counts
template <int BASIS>
__global__ void __launch_bounds__(128) km_g2p(MCtx A) {
    EP_ACTIVE(A.ctl);
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    unsigned vm0 = 0u, vm1 = 0u;
    if (c < A.g.ncell) {
        const int b = A.S.start[cur][c], e = A.S.start[cur][c + 1];
        if (b < e) {
            const int ex = c / A.g.nel[1], ez = c - ex * A.g.nel[1];
            const Axis4 ax = axis4(A.g, 0, ex), az = axis4(A.g, 1, ez);
            const double axe = A.g.ax[0][ex], aze = A.g.ax[1][ez];
            const double dt = A.ctl->dt;
            const float dtf = (float)dt, Cpf = (float)A.cf.Cpf;
            const bool musl = A.cf.musl;
            int nid[16];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    nid[j + 4 * i] = (ax.cls[i] >= 0 && az.cls[j] >= 0) ? node2(A.g, ax, az, i, j) : -1;
            float pmx[16], pmz[16];
#pragma unroll
            for (int s = 0; s < 16; ++s) pmx[s] = pmz[s] = 0.f;
            bool bad = false;
            const double ih0 = 1.0 / A.g.h[0], ih1 = 1.0 / A.g.h[1];
            for (int k = b; k < e; ++k) {
                const int p = A.S.list[cur][k];
                float wx[4], dwx[4], wz[4], dwz[4];
                point_w2<BASIS>(A, ax, az, p, cur, axe, aze, wx, dwx, wz, dwz, bad);
                float vpx = 0.f, vpz = 0.f, afx = 0.f, afz = 0.f;
#pragma unroll
                for (int s = 0; s < 16; ++s) {
                    if (nid[s] < 0) continue;
                    const float N = wx[s >> 2] * wz[s & 3];
                    vpx += N * __ldg(&A.N.v[0][nid[s]]);
                    vpz += N * __ldg(&A.N.v[1][nid[s]]);
                    afx += N * __ldg(&A.N.a[0][nid[s]]);
                    afz += N * __ldg(&A.N.a[1][nid[s]]);
                }
                const float vx = Cpf * (A.P.v[0][p] + dtf * afx) + (1.f - Cpf) * vpx;
                const float vz = Cpf * (A.P.v[1][p] + dtf * afz) + (1.f - Cpf) * vpz;
                A.P.v[0][p] = vx;
                A.P.v[1][p] = vz;
                const double xn = A.P.x[cur][0][p] + dt * (double)vpx;
                const double zn = A.P.x[cur][1][p] + dt * (double)vpz;
                A.P.x[nxt][0][p] = xn;
                A.P.x[nxt][1][p] = zn;
                vm0 = max(vm0, __float_as_uint(fabsf(vx)));
                vm1 = max(vm1, __float_as_uint(fabsf(vz)));
                // cell of the new position (clamped as in tplgy.jl:49)
                double fx = floor((xn - A.g.x0[0]) * ih0), fz = floor((zn - A.g.x0[1]) * ih1);
                int c2 = -1;
                if (isfinite(xn) && isfinite(zn)) {
                    fx = fmin(fmax(fx, 0.0), (double)(A.g.nel[0] - 1));
                    fz = fmin(fmax(fz, 0.0), (double)(A.g.nel[1] - 1));
                    c2 = (int)fz + A.g.nel[1] * (int)fx;
                    atomicAdd(&A.S.count[nxt][c2], 1);
                } else {
                    set_err(A.ctl, EP_ERR_NONFINITE, p);
                }
                A.P.p2e_next[p] = c2;
                if (musl) {
                    const float mp = A.P.mp[p];
#pragma unroll
                    for (int s = 0; s < 16; ++s) {
                        const float Nm = wx[s >> 2] * wz[s & 3] * mp;
                        pmx[s] += Nm * vx;
                        pmz[s] += Nm * vz;
                    }
                }
            }
            if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, c);
            if (musl) {
#pragma unroll
                for (int s = 0; s < 16; ++s) {
                    if (nid[s] < 0) continue;
                    atomicAdd(&A.N.pm[0][nid[s]], pmx[s]);
                    atomicAdd(&A.N.pm[1][nid[s]], pmz[s]);
                }
            }
        }
    }
    // vmax over the warp, one atomic per warp (non-negative floats order like their bits)
    vm0 = __reduce_max_sync(0xffffffffu, vm0);
    vm1 = __reduce_max_sync(0xffffffffu, vm1);
    if ((threadIdx.x & 31) == 0) {
        if (vm0) atomicMax(&A.ctl->vmax_bits[0], (unsigned long long)__double_as_longlong((double)__uint_as_float(vm0)));
        if (vm1) atomicMax(&A.ctl->vmax_bits[1], (unsigned long long)__double_as_longlong((double)__uint_as_float(vm1)));
    }
}

// km_vmusl: mUSL nodal velocity v = p/m with Dirichlet masks (augm.jl:37-53)
__global__ void km_vmusl(MCtx A) {
    EP_ACTIVE(A.ctl);
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= A.g.nnode) return;
    const float m = A.N.m[n];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        float v = 0.f;
        if (m != 0.f && !A.g.bcs[(size_t)d * A.g.nnode + n]) v = A.N.pm[d][n] * (1.f / m);
        A.N.vm[d][n] = v;
    }
}

// velocity gradient of point p from the nodal velocity field vn (deform.jl:9-10)
__device__ __forceinline__ void grad_v(const float* wx, const float* dwx, const float* wz, const float* dwz,
                                       const int* nid, float* const* vn, float* gv) {
    float g00 = 0.f, g01 = 0.f, g10 = 0.f, g11 = 0.f;
#pragma unroll
    for (int s = 0; s < 16; ++s) {
        if (nid[s] < 0) continue;
        const float Nx = dwx[s >> 2] * wz[s & 3], Nz = wx[s >> 2] * dwz[s & 3];
        const float vx = __ldg(&vn[0][nid[s]]), vz = __ldg(&vn[1][nid[s]]);
        g00 += Nx * vx;
        g01 += Nz * vx;
        g10 += Nx * vz;
        g11 += Nz * vz;
    }
    gv[0] = g00; gv[1] = g10; gv[2] = g01; gv[3] = g11;   // column-major ∇v[i + 2j] = ∂v_i/∂x_j
}

__device__ __forceinline__ void place_next(const MCtx& A, int p, int nxt) {
    const int c2 = A.P.p2e_next[p];
    if (c2 < 0) return;
    const int k = atomicAdd(&A.S.cursor[c2], 1);
    const int pos = A.S.start[nxt][c2] + k;
    if (pos < A.S.start[nxt][c2 + 1]) A.S.list[nxt][pos] = p;
    else set_err(A.ctl, EP_ERR_CUDA, p);
}

// km_fbar: δJ = det(I + dt ∇v) - 1 of every point and its P2G Σ N m δJ; builds
// the next step's cell lists (placement after the scan of the counts)
template <int BASIS>
__global__ void __launch_bounds__(128) km_fbar(MCtx A) {
    EP_ACTIVE(A.ctl);
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.g.ncell) return;
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int b = A.S.start[cur][c], e = A.S.start[cur][c + 1];
    if (b == e) return;
    const int ex = c / A.g.nel[1], ez = c - ex * A.g.nel[1];
    const Axis4 ax = axis4(A.g, 0, ex), az = axis4(A.g, 1, ez);
    const double axe = A.g.ax[0][ex], aze = A.g.ax[1][ez];
    const float dtf = (float)A.ctl->dt;
    int nid[16];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) nid[j + 4 * i] = (ax.cls[i] >= 0 && az.cls[j] >= 0) ? node2(A.g, ax, az, i, j) : -1;
    float acc[16];
#pragma unroll
    for (int s = 0; s < 16; ++s) acc[s] = 0.f;
    bool bad = false;
    float* const* vn = A.cf.musl ? A.N.vm : A.N.v;
    for (int k = b; k < e; ++k) {
        const int p = A.S.list[cur][k];
        float wx[4], dwx[4], wz[4], dwz[4];
        point_w2<BASIS>(A, ax, az, p, cur, axe, aze, wx, dwx, wz, dwz, bad);
        float gv[4];
        grad_v(wx, dwx, wz, dwz, nid, vn, gv);
        const float D00 = dtf * gv[0], D10 = dtf * gv[1], D01 = dtf * gv[2], D11 = dtf * gv[3];
        const float dJ = D00 + D11 + (D00 * D11 - D01 * D10);
        // numerator mass ρΩ after the deformation update: finite ρ0Ω0 (unchanged), infinitesimal
        // ρ J Ω0 = m (1 + δJ), so the nodal sum carries m (1+δJ)^2 - m = m δJ (2 + δJ) (volumetric.jl:8)
        const float mdj = A.P.mp[p] * (A.cf.deform == EP_DEFORM_FINITE ? dJ : dJ * (2.f + dJ));
#pragma unroll
        for (int s = 0; s < 16; ++s) acc[s] += wx[s >> 2] * wz[s & 3] * mdj;
        place_next(A, p, nxt);
    }
#pragma unroll
    for (int s = 0; s < 16; ++s)
        if (nid[s] >= 0) atomicAdd(&A.N.dJacc[nid[s]], acc[s]);
}

// km_dJn: nodal δJ_n = Σ N m δJ / m_n (volumetric.jl:12-22, increment form)
__global__ void km_dJn(MCtx A) {
    EP_ACTIVE(A.ctl);
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= A.g.nnode) return;
    const float m = A.N.m[n];
    A.N.dJn[n] = (m == 0.f) ? 0.f : A.N.dJacc[n] / m;
}

// FP32 Drucker-Prager (DP.jl:33-98) on Voigt stress s[3]; returns Δλ and its ϵpII increment
__device__ __forceinline__ float dp32(float* s, float ep2, float c0, float cr, float tphi, float Hp, float Kc, float Gc,
                                      float* dep) {
    float coh = c0 + Hp * ep2;
    if (coh < cr) coh = cr;
    const float P = 0.5f * (s[0] + s[1]);
    const float t0 = s[0] - P, t1 = s[1] - P, t2 = s[2];
    const float tII = sqrtf(0.5f * (t0 * t0 + t1 * t1) + t2 * t2);
    const float den = sqrtf(9.f + 12.f * tphi * tphi);
    const float eta = 3.f * tphi / den, xi = 3.f * coh / den;
    const float sm = xi / eta, tP = xi - eta * sm;
    const float fs = tII + eta * P - xi;
    const float h = tII - tP - sqrtf(1.f + eta * eta) * (P - sm);
    float dl = 0.f;
    *dep = 0.f;
    if ((fs > 0.f && P < sm) || (h > 0.f && P >= sm)) {
        dl = fs / Gc;                                  // ψ = 0: ηB = 0
        const float tn = xi - eta * P, r = tn / tII;
        s[0] = t0 * r + P;
        s[1] = t1 * r + P;
        s[2] = t2 * r;
        *dep = dl * 0.57735026918962576f;              // sqrt(1/3)
    }
    if (h <= 0.f && P >= sm) {
        dl = (P - sm) / Kc;
        const float Pn = sm - P, r = 0.f / tII;
        s[0] = t0 * r + Pn;
        s[1] = t1 * r + Pn;
        s[2] = t2 * r;
        *dep = 1.41421356237309505f * dl / 3.f;
    }
    return dl;
}

// FP32 J2 cutting plane (J2.jl:21-76 restated as in ep_scalar.h), 2d
__device__ __forceinline__ int j232(float* s, float ep2, float c0, float cr, float Hp, const float* D, float* g) {
    auto yield = [&](const float* v, float kap, float* n) {
        const float P = 0.5f * (v[0] + v[1]);
        const float x0 = v[0] - P, x1 = v[1] - P, x2 = v[2];
        const float xn = sqrtf(2.f * (0.5f * (x0 * x0 + x1 * x1 + 2.f * x2 * x2)));
        n[0] = x0 / xn; n[1] = x1 / xn; n[2] = x2 / xn;
        return xn - kap;
    };
    float kap = fmaxf(cr, c0 + Hp * ep2), n[3];
    float f = yield(s, kap, n);
    if (!(f > 0.f)) return 0;
    float g0 = ep2;
    for (int it = 1; fabsf(f) > 1.0e-9f && it < 20; ++it) {
        float row[3];
        for (int j = 0; j < 3; ++j) row[j] = n[0] * D[3 * j] + n[1] * D[1 + 3 * j] + n[2] * D[2 + 3 * j];
        const float dl = f / (row[0] * n[0] + row[1] * n[1] + row[2] * n[2]);
        for (int i = 0; i < 3; ++i) s[i] -= dl * (D[i] * n[0] + D[i + 3] * n[1] + D[i + 6] * n[2]);
        g0 += dl;
        kap = fmaxf(cr, c0 + Hp * g0);
        f = yield(s, kap, n);
    }
    *g = g0;
    return 1;
}

// atanh(x)/x from x² (even series for small x)
__device__ __forceinline__ float atanh_over_x(float x2) {
    if (x2 < 1.0e-3f) return 1.f + x2 * (1.f / 3.f + x2 * (1.f / 5.f + x2 * (1.f / 7.f)));
    const float x = sqrtf(x2);
    return 0.5f * (log1pf(x) - log1pf(-x)) / x;
}

// km_cons: F-bar scaling, F update, elastic predictor and return map, point by point
template <int BASIS>
__global__ void __launch_bounds__(128) km_cons(MCtx A, int plastic_phase) {
    EP_ACTIVE(A.ctl);
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.g.ncell) return;
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int b = A.S.start[cur][c], e = A.S.start[cur][c + 1];
    if (b == e) return;
    const int ex = c / A.g.nel[1], ez = c - ex * A.g.nel[1];
    const Axis4 ax = axis4(A.g, 0, ex), az = axis4(A.g, 1, ez);
    const double axe = A.g.ax[0][ex], aze = A.g.ax[1][ez];
    const float dtf = (float)A.ctl->dt;
    int nid[16];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) nid[j + 4 * i] = (ax.cls[i] >= 0 && az.cls[j] >= 0) ? node2(A.g, ax, az, i, j) : -1;
    bool bad = false;
    float* const* vn = A.cf.musl ? A.N.vm : A.N.v;
    const bool fin = A.cf.deform == EP_DEFORM_FINITE, lock = A.cf.locking;
    int nplastic = 0;
    for (int k = b; k < e; ++k) {
        const int p = A.S.list[cur][k];
        float wx[4], dwx[4], wz[4], dwz[4];
        point_w2<BASIS>(A, ax, az, p, cur, axe, aze, wx, dwx, wz, dwz, bad);
        float gv[4];
        grad_v(wx, dwx, wz, dwz, nid, vn, gv);
        // D = ΔF - I (deform.jl:13)
        float D[4] = {dtf * gv[0], dtf * gv[1], dtf * gv[2], dtf * gv[3]};
        if (A.cf.trsfr == EP_TRSFR_TPIC)
            for (int q = 0; q < 4; ++q) A.P.dv[q][p] = gv[q];
        // F <- ΔF F with the unscaled ΔF (deform.jl:14); increment in FP32, sum in FP64
        {
            double F0 = A.P.F[0][p], F1 = A.P.F[1][p], F2 = A.P.F[2][p], F3 = A.P.F[3][p];
            const float f0 = (float)F0, f1 = (float)F1, f2 = (float)F2, f3 = (float)F3;
            A.P.F[0][p] = F0 + (double)(D[0] * f0 + D[2] * f1);
            A.P.F[1][p] = F1 + (double)(D[1] * f0 + D[3] * f1);
            A.P.F[2][p] = F2 + (double)(D[0] * f2 + D[2] * f3);
            A.P.F[3][p] = F3 + (double)(D[1] * f2 + D[3] * f3);
            if (!fin) {
                // infinitesimal: the mass ρ0 J Ω0 and volume J Ω0 follow J (deform.jl:41-43)
                const double J = A.P.F[0][p] * A.P.F[3][p] - A.P.F[2][p] * A.P.F[1][p];
                const float Om = (float)(J * (double)A.P.Om0[p]);
                A.P.Om[p] = Om;
                A.P.mp[p] = A.P.rho[p] * Om;        // ρΩ with ρ fixed (the reference's infinitesimal mass)
            }
        }
        // F-bar: ΔF <- (ΔJ̄/ΔJ)^(1/2) ΔF, with ΔJ̄ = Σ N ΔJ_n (volumetric.jl:23-36)
        if (lock) {
            const float dJp = D[0] + D[3] + (D[0] * D[3] - D[2] * D[1]);
            float a = 0.f;
#pragma unroll
            for (int s = 0; s < 16; ++s)
                if (nid[s] >= 0) a += wx[s >> 2] * wz[s & 3] * __ldg(&A.N.dJn[nid[s]]);
            const float r1 = (a - dJp) / (1.f + dJp);           // ΔJ̄/ΔJ - 1
            const float s1 = r1 / (1.f + sqrtf(1.f + r1));      // sqrt(1 + r1) - 1
            D[0] = D[0] * (1.f + s1) + s1;
            D[1] = D[1] * (1.f + s1);
            D[2] = D[2] * (1.f + s1);
            D[3] = D[3] * (1.f + s1) + s1;
        }
        float t[3];
        if (fin) {
            // b <- ΔF b ΔF' = b + (D b + b D' + D b D') (elast.jl:49)
            double B0 = A.P.b[0][p], B1 = A.P.b[1][p], B2 = A.P.b[2][p];   // b11, b22, b12
            const float b11 = (float)B0, b22 = (float)B1, b12 = (float)B2;
            const float M00 = D[0] * b11 + D[2] * b12, M01 = D[0] * b12 + D[2] * b22;   // M = D b
            const float M10 = D[1] * b11 + D[3] * b12, M11 = D[1] * b12 + D[3] * b22;
            const float i11 = 2.f * M00 + (M00 * D[0] + M01 * D[2]);
            const float i22 = 2.f * M11 + (M10 * D[1] + M11 * D[3]);
            const float i12 = M10 + M01 + (M00 * D[1] + M01 * D[3]);
            B0 += (double)i11;
            B1 += (double)i22;
            B2 += (double)i12;
            A.P.b[0][p] = B0;
            A.P.b[1][p] = B1;
            A.P.b[2][p] = B2;
            // ε = ½ log b (elast.jl:51-52), spectral form
            const double m = 0.5 * (B0 + B1);
            const float dd = (float)(0.5 * (B0 - B1)), q = (float)B2, mf = (float)m;
            const float x2 = (dd * dd + q * q) / (mf * mf);
            const float L0 = (float)ep_log(m) + 0.5f * log1pf(-x2);
            const float kd = atanh_over_x(x2) / mf;
            const float e11 = 0.5f * (L0 + kd * dd), e22 = 0.5f * (L0 - kd * dd), e12 = 0.5f * kd * q;
            // τ = Del voigt(ε, 2) (elast.jl:54)
            const float v2 = 2.f * e12;
            t[0] = A.Del[0] * e11 + A.Del[3] * e22 + A.Del[6] * v2;
            t[1] = A.Del[1] * e11 + A.Del[4] * e22 + A.Del[7] * v2;
            t[2] = A.Del[2] * e11 + A.Del[5] * e22 + A.Del[8] * v2;
        } else {
            // σ += Del voigt(sym(ΔF) - I, 2) (+ ωσ - σω for the objective rate) (elast.jl:73-78)
            t[0] = A.P.tau[0][p]; t[1] = A.P.tau[1][p]; t[2] = A.P.tau[2][p];
            const float e11 = D[0], e22 = D[3], g12 = D[1] + D[2];
            float d0 = A.Del[0] * e11 + A.Del[3] * e22 + A.Del[6] * g12;
            float d1 = A.Del[1] * e11 + A.Del[4] * e22 + A.Del[7] * g12;
            float d2 = A.Del[2] * e11 + A.Del[5] * e22 + A.Del[8] * g12;
            if (A.cf.jaumann) {
                const float w = 0.5f * (D[2] - D[1]);                 // ω12
                d0 += 2.f * w * t[2];
                d1 -= 2.f * w * t[2];
                d2 += w * (t[1] - t[0]);
            }
            t[0] += d0; t[1] += d1; t[2] += d2;
        }
        if (plastic_phase) {
            const double ep1 = A.P.ep1[p];
            const float ep2 = A.cf.nonloc ? A.P.ep2[p] : (float)ep1;
            if (A.cf.cons == EP_CONS_DP) {
                float dep;
                const float dl = dp32(t, ep2, A.P.c0[p], A.P.cr[p], A.P.tphi[p], A.Hp, A.Kc, A.Gc, &dep);
                A.P.dlam[p] = dl;
                if (dl != 0.f) {
                    ++nplastic;
                    A.P.ep1[p] = ep1 + (double)dep;
                    if (fin) {
                        // ε = tensor(Del \ τ, ½); b = exp(2ε) (DP.jl:63-66), spectral form
                        const float e11 = A.Cmp[0] * t[0] + A.Cmp[3] * t[1] + A.Cmp[6] * t[2];
                        const float e22 = A.Cmp[1] * t[0] + A.Cmp[4] * t[1] + A.Cmp[7] * t[2];
                        const float e12 = 0.5f * (A.Cmp[2] * t[0] + A.Cmp[5] * t[1] + A.Cmp[8] * t[2]);
                        const float em = 0.5f * (e11 + e22), ed = 0.5f * (e11 - e22);
                        const float s2 = ed * ed + e12 * e12;
                        float ch, shs;   // cosh(2s), sinh(2s)/s
                        if (s2 < 1.0e-4f) {
                            ch = 1.f + s2 * (2.f + s2 * (2.f / 3.f));
                            shs = 2.f * (1.f + s2 * (2.f / 3.f + s2 * (2.f / 15.f)));
                        } else {
                            const float s = sqrtf(s2);
                            ch = coshf(2.f * s);
                            shs = sinhf(2.f * s) / s;
                        }
                        const double E = ep_exp(2.0 * (double)em);
                        A.P.b[0][p] = E * (double)(ch + shs * ed);
                        A.P.b[1][p] = E * (double)(ch - shs * ed);
                        A.P.b[2][p] = E * (double)(shs * e12);
                    }
                }
            } else {
                float g;
                const float Dl[9] = {A.Del[0], A.Del[1], A.Del[2], A.Del[3], A.Del[4], A.Del[5], A.Del[6], A.Del[7], A.Del[8]};
                if (j232(t, ep2, A.P.c0[p], A.P.cr[p], A.Hp, Dl, &g)) {
                    A.P.ep1[p] = (double)g;
                    if (fin) {
                        const float e11 = A.Cmp[0] * t[0] + A.Cmp[3] * t[1] + A.Cmp[6] * t[2];
                        const float e22 = A.Cmp[1] * t[0] + A.Cmp[4] * t[1] + A.Cmp[7] * t[2];
                        const float e12 = 0.5f * (A.Cmp[2] * t[0] + A.Cmp[5] * t[1] + A.Cmp[8] * t[2]);
                        const float em = 0.5f * (e11 + e22), ed = 0.5f * (e11 - e22);
                        const float s2 = ed * ed + e12 * e12;
                        const float s = sqrtf(s2);
                        const float ch = coshf(2.f * s), shs = s2 > 0.f ? sinhf(2.f * s) / s : 2.f;
                        const double E = ep_exp(2.0 * (double)em);
                        A.P.b[0][p] = E * (double)(ch + shs * ed);
                        A.P.b[1][p] = E * (double)(ch - shs * ed);
                        A.P.b[2][p] = E * (double)(shs * e12);
                    }
                }
            }
        }
        A.P.tau[0][p] = t[0];
        A.P.tau[1][p] = t[1];
        A.P.tau[2][p] = t[2];
        if (!(isfinite(t[0]) && isfinite(t[1]) && isfinite(t[2]))) set_err(A.ctl, EP_ERR_NONFINITE, p);
        if (!lock) place_next(A, p, nxt);
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, c);
    if (nplastic) atomicAdd((unsigned long long*)&A.ctl->plastic, (unsigned long long)nplastic);
}

__global__ void km_flip(Ctl* ctl) {
    if (ctl->active) ctl->parity ^= 1;
}

// ---------------------------------------------------------------------------
// import / export between the FP64 staging layout (P64, the reference's
// arrays in SoA) and the mixed state
__global__ void km_import(MCtx A, P64 Q, int with_topology) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.P.np) return;
    const int cur = A.ctl->parity;
    for (int d = 0; d < 2; ++d) {
        A.P.x[cur][d][p] = Q.x[d][p];
        A.P.v[d][p] = (float)Q.v[d][p];
        if (A.cf.basis == EP_BASIS_GIMPM) A.P.l[d][p] = (float)Q.l[d][p];
    }
    for (int k = 0; k < 4; ++k) {
        A.P.F[k][p] = Q.F[k][p];
        if (A.cf.trsfr == EP_TRSFR_TPIC) A.P.dv[k][p] = (float)Q.dv[k][p];
    }
    A.P.b[0][p] = Q.b[0][p];
    A.P.b[1][p] = Q.b[3][p];
    A.P.b[2][p] = 0.5 * (Q.b[2][p] + Q.b[1][p]);
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    for (int k = 0; k < 3; ++k) A.P.tau[k][p] = (float)(fin ? Q.tau[k][p] : Q.sig[k][p]);
    A.P.ep1[p] = Q.ep1[p];
    A.P.ep2[p] = (float)Q.ep2[p];
    A.P.dlam[p] = (float)Q.dlam[p];
    A.P.c0[p] = (float)Q.c0[p];
    A.P.cr[p] = (float)Q.cr[p];
    A.P.tphi[p] = (float)Q.tphi[p];
    A.P.sphi[p] = (float)Q.sphi[p];
    A.P.cphi[p] = (float)Q.cphi[p];
    A.P.mp[p] = (float)(Q.rho[p] * Q.Om[p]);
    A.P.Om0[p] = (float)Q.Om0[p];
    A.P.Om[p] = (float)Q.Om[p];
    A.P.rho[p] = (float)Q.rho[p];
}

__global__ void km_export(MCtx A, P64 Q) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.P.np) return;
    const int cur = A.ctl->parity;
    for (int d = 0; d < 2; ++d) {
        Q.x[d][p] = A.P.x[cur][d][p];
        Q.v[d][p] = (double)A.P.v[d][p];
        if (A.cf.basis == EP_BASIS_GIMPM) Q.l[d][p] = (double)A.P.l[d][p];
    }
    const double F0 = A.P.F[0][p], F1 = A.P.F[1][p], F2 = A.P.F[2][p], F3 = A.P.F[3][p];
    Q.F[0][p] = F0; Q.F[1][p] = F1; Q.F[2][p] = F2; Q.F[3][p] = F3;
    const double J = F0 * F3 - F2 * F1;
    Q.J[p] = J;
    Q.Om[p] = J * Q.Om0[p];
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    if (fin) {
        Q.rho[p] = Q.rho0[p] / J;
        Q.n[p] = 1.0 - 1.0 / J * (1.0 - Q.n0[p]);
        const double B0 = A.P.b[0][p], B1 = A.P.b[1][p], B2 = A.P.b[2][p];
        Q.b[0][p] = B0; Q.b[3][p] = B1; Q.b[1][p] = B2; Q.b[2][p] = B2;
        for (int k = 0; k < 3; ++k) {
            Q.tau[k][p] = (double)A.P.tau[k][p];
            Q.sig[k][p] = (double)A.P.tau[k][p] / J;
        }
        // ϵ = ½ log b (FP64, for output)
        double lam[2], V[4], L[2], R[4];
        eig_sym2(B0, B2, B1, lam, V);
        L[0] = ep_log(lam[0]);
        L[1] = ep_log(lam[1]);
        vdvt<2>(V, L, R);
        for (int k = 0; k < 4; ++k) Q.eps[k][p] = 0.5 * R[k];
    } else {
        for (int k = 0; k < 3; ++k) Q.sig[k][p] = (double)A.P.tau[k][p];
    }
    if (A.cf.trsfr == EP_TRSFR_TPIC)
        for (int k = 0; k < 4; ++k) Q.dv[k][p] = (double)A.P.dv[k][p];
    Q.ep1[p] = A.P.ep1[p];
    Q.ep2[p] = A.cf.nonloc ? (double)A.P.ep2[p] : A.P.ep1[p];
    Q.dlam[p] = (double)A.P.dlam[p];
    // element of the current position (for p2e/p2n on download)
    const double fx = floor((Q.x[0][p] - A.g.x0[0]) / A.g.h[0]), fz = floor((Q.x[1][p] - A.g.x0[1]) / A.g.h[1]);
    int c2 = -1;
    if (fx == fx && fz == fz)
        c2 = (int)fmin(fmax(fz, 0.0), (double)(A.g.nel[1] - 1)) +
             A.g.nel[1] * (int)fmin(fmax(fx, 0.0), (double)(A.g.nel[0] - 1));
    Q.p2e[p] = c2;
}

__global__ void km_export_nodes(MCtx A, N64 Q) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= A.g.nnode) return;
    Q.m[n] = A.N.m[n];
    for (int d = 0; d < 2; ++d) {
        Q.p[d][n] = A.cf.musl ? A.N.pm[d][n] : A.N.p[d][n];
        Q.v[d][n] = A.cf.musl ? A.N.vm[d][n] : A.N.v[d][n];
        Q.a[d][n] = A.N.a[d][n];
        Q.oobf[d][n] = A.N.f[d][n];
    }
    Q.dJ[n] = 1.0 + (double)A.N.dJn[n];
}

// initial cell lists (positions of the current buffer)
__global__ void km_bin0(MCtx A) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.P.np) return;
    const int cur = A.ctl->parity;
    const double fx = floor((A.P.x[cur][0][p] - A.g.x0[0]) / A.g.h[0]);
    const double fz = floor((A.P.x[cur][1][p] - A.g.x0[1]) / A.g.h[1]);
    int c2 = -1;
    if (isfinite(A.P.x[cur][0][p]) && isfinite(A.P.x[cur][1][p])) {
        c2 = (int)fmin(fmax(fz, 0.0), (double)(A.g.nel[1] - 1)) +
             A.g.nel[1] * (int)fmin(fmax(fx, 0.0), (double)(A.g.nel[0] - 1));
        atomicAdd(&A.S.count[cur][c2], 1);
    } else {
        set_err(A.ctl, EP_ERR_NONFINITE, p);
    }
    A.P.p2e_next[p] = c2;
}

__global__ void km_place0(MCtx A) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.P.np) return;
    place_next(A, p, A.ctl->parity);
}

// ---------------------------------------------------------------------------
template <int BASIS>
static void mixed_step_impl(const MixedCtx& X, int phase, cudaStream_t s) {
    const MCtx& A = *(const MCtx*)X.impl;
    const int nc = A.g.ncell, nn = A.g.nnode;
    const int TB = 128;
    const int gc = (nc + TB - 1) / TB, gn = (nn + TB - 1) / TB;
    Prof* pr = (X.prof && X.prof->on) ? X.prof : nullptr;
    auto mark = [&](const char* nm) {
        if (pr) pr->mark(nm, s);
    };
    // grid accumulators of this step and next-step counters (one contiguous block each)
    cudaMemsetAsync(X.grid_zero, 0, X.grid_zero_bytes, s);
    cudaMemsetAsync(X.sort_zero, 0, X.sort_zero_bytes, s);   // both parities' counts and the cursor
    mark("memset");
    km_p2g<BASIS><<<gc, TB, 0, s>>>(A);
    mark("p2g");
    km_solve<<<gn, TB, 0, s>>>(A);
    mark("solve");
    km_g2p<BASIS><<<gc, TB, 0, s>>>(A);
    mark("g2p");
    if (A.cf.musl) { km_vmusl<<<gn, TB, 0, s>>>(A); mark("vmusl"); }
    launch_mixed_scan(X, s);
    mark("scan");
    if (A.cf.locking) {
        km_fbar<BASIS><<<gc, TB, 0, s>>>(A);
        mark("fbar");
        km_dJn<<<gn, TB, 0, s>>>(A);
        mark("dJn");
    }
    km_cons<BASIS><<<gc, TB, 0, s>>>(A, phase == EP_PHASE_ELASTOPLASTIC);
    mark("cons");
    km_flip<<<1, 1, 0, s>>>(A.ctl);
    if (X.launches) *X.launches += 5 + 2 + (nc > 4096 ? 3 : 2) + (A.cf.musl ? 1 : 0) + (A.cf.locking ? 2 : 0);
}

void mixed_step(const MixedCtx& X, int phase, cudaStream_t s) {
    const MCtx& A = *(const MCtx*)X.impl;
    if (A.cf.basis == EP_BASIS_BSMPM) mixed_step_impl<EP_BASIS_BSMPM>(X, phase, s);
    else if (A.cf.basis == EP_BASIS_GIMPM) mixed_step_impl<EP_BASIS_GIMPM>(X, phase, s);
    else mixed_step_impl<EP_BASIS_SMPM>(X, phase, s);
}

// exclusive scan of the next-parity counts into the next-parity starts; the
// parity lives on the device, so scan both candidate buffers' roles through a
// tiny selector kernel: copy counts[nxt] to the scan input first
__global__ void km_sel_counts(MCtx A, int* dst) {
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A.g.ncell) dst[i] = A.ctl->active ? A.S.count[nxt][i] : 0;
}
__global__ void km_put_starts(MCtx A, const int* src) {
    if (!A.ctl->active) return;
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= A.g.ncell) A.S.start[nxt][i] = src[i];
}

void launch_mixed_scan(const MixedCtx& X, cudaStream_t s) {
    const MCtx& A = *(const MCtx*)X.impl;
    const int nc = A.g.ncell;
    km_sel_counts<<<(nc + 255) / 256, 256, 0, s>>>(A, X.scan_in);
    launch_exclusive_scan(X.scan_in, X.scan_out, nc, A.S.scan_tmp, s);
    km_put_starts<<<(nc + 256) / 256, 256, 0, s>>>(A, X.scan_out);
}

void mixed_import(const MixedCtx& X, const P64& Q, cudaStream_t s) {
    const MCtx& A = *(const MCtx*)X.impl;
    const int np = A.P.np;
    if (np > 0) km_import<<<(np + 255) / 256, 256, 0, s>>>(A, Q, 0);
    // initial cell lists for the current parity
    cudaMemsetAsync(X.sort_zero, 0, X.sort_zero_bytes, s);
    if (np > 0) km_bin0<<<(np + 255) / 256, 256, 0, s>>>(A);
    // scan counts[cur] -> start[cur]
    mixed_initial_scan(X, s);
    if (np > 0) km_place0<<<(np + 255) / 256, 256, 0, s>>>(A);
}

__global__ void km_sel_counts_cur(MCtx A, int* dst) {
    const int cur = A.ctl->parity;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A.g.ncell) dst[i] = A.S.count[cur][i];
}
__global__ void km_put_starts_cur(MCtx A, const int* src) {
    const int cur = A.ctl->parity;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= A.g.ncell) A.S.start[cur][i] = src[i];
}

void mixed_initial_scan(const MixedCtx& X, cudaStream_t s) {
    const MCtx& A = *(const MCtx*)X.impl;
    const int nc = A.g.ncell;
    km_sel_counts_cur<<<(nc + 255) / 256, 256, 0, s>>>(A, X.scan_in);
    launch_exclusive_scan(X.scan_in, X.scan_out, nc, A.S.scan_tmp, s);
    km_put_starts_cur<<<(nc + 256) / 256, 256, 0, s>>>(A, X.scan_out);
}

void mixed_export(const MixedCtx& X, const P64& Q, const N64& QN, cudaStream_t s) {
    const MCtx& A = *(const MCtx*)X.impl;
    const int np = A.P.np;
    if (np > 0) km_export<<<(np + 255) / 256, 256, 0, s>>>(A, Q);
    km_export_nodes<<<(A.g.nnode + 255) / 256, 256, 0, s>>>(A, QN);
}

// host-side construction of the device context
size_t mixed_ctx_size() { return sizeof(MCtx); }

void mixed_ctx_init(void* mem, const Cfg& cf, const Geo& g, Ctl* ctl, const PM& P, const NM& N, const SM& S,
                    const double* Del, const double* Cmp, double Kc, double Gc, double Hp, double c) {
    MCtx* A = (MCtx*)mem;
    A->cf = cf;
    A->g = g;
    A->ctl = ctl;
    A->P = P;
    A->N = N;
    A->S = S;
    for (int i = 0; i < 9; ++i) {
        A->Del[i] = (float)Del[i];
        A->Cmp[i] = (float)Cmp[i];
    }
    A->Kc = (float)Kc;
    A->Gc = (float)Gc;
    A->Hp = (float)Hp;
    A->c = c;
}

}  // namespace ep
