// ep_mixed.cu -- the mixed-precision MPM steps (2d), the fast path.
//
// Same method and call order as the reference step (worflow.jl:80-82); the
// transfers and the grid arithmetic run in FP32.  What needs more than FP32
// is kept in a wider accumulator:
//   * the accumulated kinematic state F, b_e and the accumulated plastic
//     strain: FP64 ("mixed", ACC = 0) or double-float pairs of FP32 values
//     ("mixed_df", ACC = 1; GB300 issues FP64 at 1/64 of the FP32 rate, and a
//     pair carries 48 significand bits with FP32 instructions only).  Their
//     per-step increments are small (dt∇v ~ 1e-4) and formed in FP32;
//   * positions: FP32 offsets from the left node of the point's cell
//     (|offset| < h, so an FP32 ulp is ~1e-7 h); the cell index is exact;
//   * F-bar carries δJ = ΔJ - 1 instead of ΔJ (volumetric.jl:1-36 in
//     increment form), so nothing cancels against 1 in FP32;
//   * log b_e and exp(2ε) (elast.jl:49-54, DP.jl:63-66) use the closed
//     spectral form of a symmetric 2x2 tensor A = m I + A_d (eigenvalues m ± r):
//       log A = (log m + ½ log(1 - x²)) I + (atanh(x)/x)/m · A_d,  x = r/m,
//       exp(2E) = e^{2 e_m} (cosh(2s) I + sinh(2s)/s · E_d),       s² = ½ tr(E_d²);
//     the isotropic part (log m, e^{2 e_m}) is FP64 for ACC = 0 and, for
//     ACC = 1, log1p/expm1 of the deviation from 1 formed exactly from the
//     double-float state; the deviatoric factors are FP32 functions of the
//     small invariants x², s².
//
// Kernels of one 2d step (t = cells staged per CTA tile, p = one lane per sorted point, n = node):
//   km_p2g_tile   P2G of m, p, f; 4 lanes per cell own its 4 stencil columns  (p2n.jl:135-155, 217-240)  t
//   km_solve      grid update                                                (solve.jl:14-40)           n
//   km_g2p_seg    PIC/FLIP, positions, vmax, next-cell counts; TPIC's ∇v or APIC's Bᵢⱼ
//                 (n2p.jl:14-40, tplgy.jl:43-62, Bij.jl:14-26)                                          p
//   km_aux_tile   mUSL momentum P2G in the tile form                         (augm.jl:13-25)            t
//   km_vmusl      mUSL nodal velocity                                        (augm.jl:37-53)            n
//   km_scan_*     next-step cell offsets (exclusive scan of the counts)
//   km_fbar_seg   ∇v, δJ and Σ N m δJ; next-step cell lists                  (deform.jl:9-18,
//                 volumetric.jl:1-11)                                                                   p
//   km_dJn        nodal δJ                                                   (volumetric.jl:12-22)      n
//   km_cons       F-bar, F, GIMP domain, elastic predictor, DP/J2            (volumetric.jl:23-36,
//                 deform.jl, domain.jl, elast.jl, DP.jl, J2.jl)                                         p
// The 3d step has the same sequence (km_p2g_tile3, km_g2p_seg3, km_fbar_seg3, km_cons3).  In a tile,
// the lanes of one cell own disjoint stencil columns, so they never add to the same node and keep
// their columns' sums in registers: one FP32 atomic per node and quantity per cell reaches the grid
// (or, in the deterministic mode, one store into the cell's node partials).
#include <climits>
#include <cstdlib>
#include <type_traits>

#include "../../include/epgpu.h"
#include "ep_internal.h"
#include "ep_mixed.cuh"
#include "ep_rmap.h"

namespace ep {

#define EP_ACTIVE(ctl) \
    if (!(ctl)->active) return

// Programmatic dependent launch (the kernels of the 2d step, launched by launch_pdl): a kernel may be
// scheduled while its predecessor in the stream drains.  Each such kernel calls pdl_enter() before
// its first memory access: griddepcontrol.wait returns once the preceding kernel has completed and
// its writes are visible, and launch_dependents then lets the following kernel's blocks be
// scheduled.  Every block executes both, so no kernel of the chain completes before its predecessor.
// In a kernel launched without the attribute both instructions do nothing.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

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
// offset dloc = x - x_e (x_e: node e, the left node of the point's cell).
// Cells whose 4 stencil nodes are all interior B-spline nodes use the
// uniform cubic B-spline in closed form (the t3 piece of bsmpm.jl:32-48
// evaluated at ξ = f+1, f, f-1, f-2 with f = dloc/h).
template <int BASIS>
__device__ __forceinline__ void axis_w(const Axis4& a, float dloc, float h, float ih, float lp, float* w, float* dw,
                                       bool& bad) {
    if (BASIS == EP_BASIS_BSMPM && a.cls[0] == BS_T3 && a.cls[1] == BS_T3 && a.cls[2] == BS_T3 && a.cls[3] == BS_T3) {
        const float f = dloc * ih, g = 1.f - f;
        const float f2 = f * f, g2 = g * g;
        w[0] = (1.f / 6.f) * g2 * g;
        w[1] = (0.5f * f - 1.f) * f2 + (2.f / 3.f);
        w[2] = (0.5f * g - 1.f) * g2 + (2.f / 3.f);
        w[3] = (1.f / 6.f) * f2 * f;
        dw[0] = -0.5f * g2 * ih;
        dw[1] = (1.5f * f - 2.f) * f * ih;
        dw[2] = (2.f - 1.5f * g) * g * ih;
        dw[3] = 0.5f * f2 * ih;
        return;
    }
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

// GIMP weight the stencil loses to nodes outside the grid along one direction (GIMP
// and the linear hat sum to one on the full line; the B-spline boundary pieces sum to one
// inside the mesh): the F-bar average Σ N ΔJ_n runs over the existing nodes only
// (volumetric.jl:23-36), so Σ N - 1 = Π_d (1 - miss_d) - 1 enters its increment form
template <int BASIS>
__device__ __forceinline__ float axis_miss(const Axis4& a, float dloc, float h, float lp) {
    float m = 0.f;
    if (BASIS == EP_BASIS_GIMPM) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (a.cls[k] < 0) {
                float f, df;
                gimp32(dloc + h * (float)(1 - k), h, lp, f, df);
                m += f;
            }
    }
    return m;
}

struct MCtx {
    Cfg cf;
    Geo g;
    Ctl* ctl;
    PM P;
    NM N;
    SM S;
    float Del[36];      // FP32 copy of the nstr x nstr stiffness (3x3 in 2d, 6x6 in 3d), column-major
    float Cmp[36];      // its inverse (compliance), FP32
    float Kc, Gc, Hp;
    double c;           // wave speed
    int acc;            // 0: FP64 accumulators, 1: double-float accumulators
    // return map (EP_RMAP_*): learned-mode slots or the record buffer
    int rmode;
    float l2g;          // λ / (2G)
    float *rx, *ry, *raux;
    int* rpt;
    int* rcount;
    int* fbcount;       // learned mode: slots the network's output was rejected for
    int* fblist;
    long long* rec_count;
    long long rec_cap;
    double Deld[36], Cmpd[36], Kd, Gd;   // FP64 copies for the exact fallback
    double DelLU[36];   // LU factors of the FP64 Del (pivots in piv) for the MC and Cam-Clay returns
    int piv[6];
    // deterministic mode: per-cell node partials (ncell x 16 x up to 5) and a per-point value
    float* part;
    float* ptmp;
};

__device__ __forceinline__ int node2(const Geo& g, const Axis4& ax, const Axis4& az, int i, int j) {
    return (az.base + j) + g.nno[1] * (ax.base + i);
}

// four lanes per cell; lane q owns stencil column q
struct Quad {
    int c, q, b, e, ex, ez;
    bool live;
};

__device__ __forceinline__ Quad quad_of(const MCtx& A, int cur) {
    Quad Q;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    Q.c = t >> 2;
    Q.q = t & 3;
    Q.live = Q.c < A.g.ncell;
    Q.b = Q.e = 0;
    Q.ex = Q.ez = 0;
    if (Q.live) {
        Q.b = A.S.start[cur][Q.c];
        Q.e = A.S.start[cur][Q.c + 1];
        Q.ex = Q.c / A.g.nel[1];
        Q.ez = Q.c - Q.ex * A.g.nel[1];
    }
    return Q;
}

// ---------------------------------------------------------------------------
// The grid update of one node (solve.jl:14-40): from its mass m, momentum p and force f, the damped
// force (f, in place), the acceleration a and the velocity v; a direction with bit d of bc set
// (Dirichlet) keeps a = v = 0 and its force undamped.  f has three entries (0 beyond D).
__device__ __forceinline__ void grid_update(int D, float m, const float* p, float* f, int bc, float dt, float eta,
                                            float* a, float* v) {
    for (int d = 0; d < 3; ++d) a[d] = v[d] = 0.f;
    if (m == 0.f) return;
    const float mi = 1.f / m;
    for (int d = 0; d < D; ++d) {
        if ((bc >> d) & 1) continue;
        // the norm sees the components damped so far (solve.jl:29)
        const float nrm = sqrtf(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
        const float pv = p[d] * mi;
        const float sg = pv > 0.f ? 1.f : (pv < 0.f ? -1.f : 0.f);
        if (fabsf(pv) >= 1.0e-3f) f[d] -= eta * nrm * sg;
        a[d] = f[d] * mi;
        v[d] = (p[d] + dt * f[d]) * mi;
    }
}

// km_solve: the grid update of every node, 2d and 3d.  N.f keeps the undamped P2G force (the
// export forms the damped one with grid_update); the mUSL accumulators are zeroed for the G2P.
__device__ __forceinline__ void solve_body(const MCtx& A, int bid) {
    EP_ACTIVE(A.ctl);
    const int n = bid * blockDim.x + threadIdx.x;
    if (n >= A.g.nnode) return;
    const int D = A.g.dim;
    const float m = A.N.m[n];
    float a[3], v[3], f[3] = {0.f, 0.f, 0.f}, pn[3] = {0.f, 0.f, 0.f};
    if (m != 0.f) {
        for (int d = 0; d < D; ++d) {
            f[d] = A.N.f[d][n];
            pn[d] = A.N.p[d][n];
        }
    }
    grid_update(D, m, pn, f, A.g.bcw[n], (float)A.ctl->dt, (float)A.cf.damping, a, v);
    for (int d = 0; d < D; ++d) {
        A.N.a[d][n] = a[d];
        A.N.v[d][n] = v[d];
        A.N.pm[d][n] = 0.f;
    }
    A.N.dJacc[n] = 0.f;
    if (D == 2) {
        A.N.va4[n] = make_float4(v[0], v[1], a[0], a[1]);
        if (!A.cf.musl) A.N.vg4[n] = make_float4(v[0], v[1], 0.f, m != 0.f ? 1.f / m : 0.f);
    }
}

__global__ void km_solve(MCtx A) {
    pdl_enter();
    solve_body(A, blockIdx.x);
}


// new cell and offset along one direction after a move of the offset o
// (relative to node e of the old cell), clamped to the mesh like tplgy.jl:49
__device__ __forceinline__ void recell(const Geo& g, int d, int e, float o, float ih, int& e2, float& o2) {
    int k = (int)floorf(o * ih);
    e2 = min(max(e + k, 0), g.nel[d] - 1);
    o2 = o;
    if (e2 != e) o2 = o - (float)(g.ax[d][e2] - g.ax[d][e]);
}

// ---------------------------------------------------------------------------
// Point-parallel transfers over the sorted cell lists: lane = one list slot, so
// the lanes of a cell are adjacent in a warp.  A scatter sums each node's
// contributions over the lanes of the same cell with a segmented warp reduction
// (towards the first lane of the cell), and that lane issues one FP32 atomic
// per node and quantity.  Gathers read the cell's 16 nodes through L1.
struct Seg {
    int lane, last, steps;   // last lane of this lane's cell in the warp; reduction steps
    bool head;               // first lane of its cell in the warp
};

// segments of equal cell ids c (c < 0: not a point)
__device__ __forceinline__ Seg seg_of(int c) {
    Seg s;
    s.lane = threadIdx.x & 31;
    const int up = __shfl_up_sync(0xffffffffu, c, 1);
    const unsigned heads = __ballot_sync(0xffffffffu, s.lane == 0 || c != up);
    s.head = (heads >> s.lane) & 1u;
    const unsigned after = s.lane == 31 ? 0u : (heads & ~((2u << s.lane) - 1u));
    s.last = after ? (__ffs(after) - 2) : 31;
    const int len = __reduce_max_sync(0xffffffffu, (unsigned)(s.last - s.lane + 1));
    s.steps = len <= 1 ? 0 : len <= 2 ? 1 : len <= 4 ? 2 : len <= 8 ? 3 : len <= 16 ? 4 : 5;
    return s;
}

// sum of v over the lanes [lane, last] of the segment (meaningful at the segment head)
__device__ __forceinline__ float seg_sum(float v, const Seg& s) {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        if (i >= s.steps) break;
        const int o = 1 << i;
        const float t = __shfl_down_sync(0xffffffffu, v, o);
        if (s.lane + o <= s.last) v += t;
    }
    return v;
}

// the point of list slot k with its cell's stencil and the shape values along both axes
struct PtW {
    int p, c, ex, ez;
    Axis4 ax, az;
    float wx[4], dwx[4], wz[4], dwz[4];
    float dx, dz;
};

template <int BASIS>
__device__ __forceinline__ bool point_of(const MCtx& A, int cur, int k, int n, PtW& W, bool& bad) {
    if (k >= n) {
        W.p = -1;
        W.c = -1;
        return false;
    }
    W.p = A.S.list[cur][k];
    W.c = A.S.cellof[cur][k];
    W.ex = W.c / A.g.nel[1];
    W.ez = W.c - W.ex * A.g.nel[1];
    W.ax = axis4(A.g, 0, W.ex);
    W.az = axis4(A.g, 1, W.ez);
    const float hx = (float)A.g.h[0], hz = (float)A.g.h[1];
    W.dx = A.P.dx[cur][0][W.p];
    W.dz = A.P.dx[cur][1][W.p];
    const float lx = BASIS == EP_BASIS_GIMPM ? A.P.l[0][W.p] : 0.f;
    const float lz = BASIS == EP_BASIS_GIMPM ? A.P.l[1][W.p] : 0.f;
    axis_w<BASIS>(W.ax, W.dx, hx, 1.f / hx, lx, W.wx, W.dwx, bad);
    axis_w<BASIS>(W.az, W.dz, hz, 1.f / hz, lz, W.wz, W.dwz, bad);
    return true;
}

// km_g2p_seg: PIC/FLIP (n2p.jl:14-40), new cell + offset, vmax, next-cell counts
// (tplgy.jl:43-62) and the mUSL momentum P2G (augm.jl:13-25), one lane per point
// MSEG: the mUSL momentum scatter by segmented warp sums here (else km_aux_tile<.., 1, ..> does it)
template <int BASIS, bool DET, bool MSEG = !DET>
__device__ __forceinline__ void g2p_seg_body(const MCtx& A, int bid) {
    EP_ACTIVE(A.ctl);
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int n = A.S.start[cur][A.g.ncell];
    const int k = bid * blockDim.x + threadIdx.x;
    bool bad = false;
    PtW W;
    const bool live = point_of<BASIS>(A, cur, k, n, W, bad);
    const Seg S = seg_of(W.c);
    const float ihx = 1.f / (float)A.g.h[0], ihz = 1.f / (float)A.g.h[1];
    const float dtf = (float)A.ctl->dt, Cpf = (float)A.cf.Cpf;
    unsigned vm0 = 0u, vm1 = 0u;
    float vx = 0.f, vz = 0.f, mp = 0.f;
    int c2 = -1;
    if (live) {
        float vpx = 0.f, vpz = 0.f, afx = 0.f, afz = 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (W.ax.cls[i] < 0) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (W.az.cls[j] < 0) continue;
                const int nd = node2(A.g, W.ax, W.az, i, j);
                const float N = W.wx[i] * W.wz[j];
                const float4 q = A.N.va4[nd];
                vpx += N * q.x;
                vpz += N * q.y;
                afx += N * q.z;
                afz += N * q.w;
            }
        }
        const int p = W.p;
        if (A.cf.trsfr == EP_TRSFR_APIC) {
            // Bᵢⱼ = Σ N v_n δᵀ, δ = node - point at the step start (Bij.jl:14-26); a pass of its own
            // so that the other transfers keep the register budget of the loop above
            const float hx = (float)A.g.h[0], hz = (float)A.g.h[1];
            float b00 = 0.f, b10 = 0.f, b01 = 0.f, b11 = 0.f;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (W.ax.cls[i] < 0) continue;
                const float dlx = (float)(i - 1) * hx - W.dx;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (W.az.cls[j] < 0) continue;
                    const float N = W.wx[i] * W.wz[j];
                    const float4 q = A.N.va4[node2(A.g, W.ax, W.az, i, j)];
                    const float dlz = (float)(j - 1) * hz - W.dz;
                    b00 += N * (q.x * dlx);
                    b10 += N * (q.y * dlx);
                    b01 += N * (q.x * dlz);
                    b11 += N * (q.y * dlz);
                }
            }
            A.P.dv[0][p] = b00;
            A.P.dv[1][p] = b10;
            A.P.dv[2][p] = b01;
            A.P.dv[3][p] = b11;
        }
        vx = Cpf * (A.P.v[0][p] + dtf * afx) + (1.f - Cpf) * vpx;
        vz = Cpf * (A.P.v[1][p] + dtf * afz) + (1.f - Cpf) * vpz;
        A.P.v[0][p] = vx;
        A.P.v[1][p] = vz;
        vm0 = __float_as_uint(fabsf(vx));
        vm1 = __float_as_uint(fabsf(vz));
        // x += dt v_PIC as a cell offset update, then re-binning (tplgy.jl:49)
        const float ox = W.dx + dtf * vpx, oz = W.dz + dtf * vpz;
        if (isfinite(ox) && isfinite(oz)) {
            int ex2, ez2;
            float o2x, o2z;
            recell(A.g, 0, W.ex, ox, ihx, ex2, o2x);
            recell(A.g, 1, W.ez, oz, ihz, ez2, o2z);
            c2 = ez2 + A.g.nel[1] * ex2;
            A.P.dx[nxt][0][p] = o2x;
            A.P.dx[nxt][1][p] = o2z;
        } else {
            set_err(A.ctl, EP_ERR_NONFINITE, p);
        }
        A.P.p2e_next[p] = c2;
        if (A.P.pcell[nxt]) A.P.pcell[nxt][p] = c2;
        mp = A.P.mp[p];
    }
    {
        // next-cell counts: one atomic per distinct cell of the warp
        const unsigned mm = __match_any_sync(0xffffffffu, c2);
        if (c2 >= 0 && S.lane == __ffs(mm) - 1) atomicAdd(&A.S.count[nxt][c2], __popc(mm));
    }
    if (A.cf.musl && MSEG) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float Nm = live ? W.wx[i] * W.wz[j] * mp : 0.f;
                const float sx = seg_sum(Nm * vx, S), sz = seg_sum(Nm * vz, S);
                if (S.head && live && W.ax.cls[i] >= 0 && W.az.cls[j] >= 0) {
                    const int nd = node2(A.g, W.ax, W.az, i, j);
                    atomicAdd(&A.N.pm[0][nd], sx);
                    atomicAdd(&A.N.pm[1][nd], sz);
                }
            }
        }
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, W.c);
    // vmax over the warp, one atomic per warp (non-negative floats order like their bits)
    vm0 = __reduce_max_sync(0xffffffffu, vm0);
    vm1 = __reduce_max_sync(0xffffffffu, vm1);
    if (S.lane == 0) {
        if (vm0) atomicMax(&A.ctl->vmax_bits[0], (unsigned long long)__double_as_longlong((double)__uint_as_float(vm0)));
        if (vm1) atomicMax(&A.ctl->vmax_bits[1], (unsigned long long)__double_as_longlong((double)__uint_as_float(vm1)));
    }
}

template <int BASIS, bool DET, bool MSEG = !DET>
__global__ void __launch_bounds__(256) km_g2p_seg(MCtx A) {
    g2p_seg_body<BASIS, DET, MSEG>(A, blockIdx.x);
}


// ---------------------------------------------------------------------------
// Shared-memory staging of a tile (the gather kernels km_g2p_tile, km_fbar_tile): a CTA owns the
// cells [c0, c1); before its first point it stages, per cell, the element indices and the node
// classes of both stencil axes (one division and eight class reads per cell instead of per point),
// and the node values its points gather, as a box of x nodes [X0, X0 + NX) by z nodes
// [Z0, Z0 + NZ): the range's own z extent when it lies in one cell column, whole columns when it
// spans several.  The box is filled with cp.async (no registers held, nodes outside the grid
// zero-filled) while the first points' list slots load.  A box above TB_MAX nodes (a range that
// wraps a column of more than ~200 cells) is not staged: the points then read the node array in
// place through the same index, with X0 = Z0 = 0 and NZ = nno_z.
constexpr int TB_MAX = 1024;

struct TileBox {
    int X0, Z0, NZ;
    bool staged;
};

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

template <int BYTES>
__device__ __forceinline__ void cp_async_zfill(void* dst, const void* src, bool valid) {
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async sizes");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(smem_addr(dst)), "l"(src), "n"(BYTES),
                 "r"(valid ? BYTES : 0)
                 : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// the box of the cells [c0, c1): x nodes [X0, X0 + NX), z nodes [Z0, Z0 + NZ) (stencils span e-1 .. e+2),
// staged when it holds at most `limit` nodes
__host__ __device__ __forceinline__ TileBox tile_box(const Geo& g, int c0, int c1, int& NX, int limit = TB_MAX) {
    TileBox b;
    const int n1 = g.nel[1];
    const int ea = c0 / n1, eb = (c1 - 1) / n1;
    b.X0 = ea - 1;
    NX = eb - ea + 4;
    if (ea == eb) {
        b.Z0 = c0 - ea * n1 - 1;
        b.NZ = (c1 - 1 - eb * n1) - (c0 - ea * n1) + 4;
    } else {
        b.Z0 = -1;
        b.NZ = n1 + 3;
    }
    b.staged = NX * b.NZ <= limit;
    if (!b.staged) {
        b.X0 = 0;
        b.Z0 = 0;
        b.NZ = g.nno[1];
    }
    return b;
}

// stage the box of V-sized leading parts of the packed node values src (stride float4)
template <typename V>
__device__ __forceinline__ void stage_box(const Geo& g, const float4* src, V* box, const TileBox& b, int NX) {
    const int n = NX * b.NZ;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int bx = 0, bz = i;
        while (bz >= b.NZ) {
            bz -= b.NZ;
            ++bx;
        }
        const int nx = b.X0 + bx, nz = b.Z0 + bz;
        const bool ok = nx >= 0 && nx < g.nno[0] && nz >= 0 && nz < g.nno[1];
        cp_async_zfill<sizeof(V)>(box + i, ok ? (const void*)(src + nz + (size_t)g.nno[1] * nx) : (const void*)src,
                                  ok);
    }
}

// per cell of the range: ex, ez and the classes of the 4 stencil nodes along x and along z
__device__ __forceinline__ void stage_cells(const Geo& g, int c0, int c1, int4* ci) {
    for (int i = threadIdx.x; i < c1 - c0; i += blockDim.x) {
        const int c = c0 + i, ex = c / g.nel[1], ez = c - ex * g.nel[1];
        const Axis4 ax = axis4(g, 0, ex), az = axis4(g, 1, ez);
        int px, pz;
        memcpy(&px, ax.cls, 4);
        memcpy(&pz, az.cls, 4);
        ci[i] = make_int4(ex, ez, px, pz);
    }
}

__device__ __forceinline__ void cell_axes(const int4& r, Axis4& ax, Axis4& az) {
    ax.base = r.x - 1;
    az.base = r.y - 1;
    memcpy(ax.cls, &r.z, 4);
    memcpy(az.cls, &r.w, 4);
}

// box index of stencil node (i, j)
__device__ __forceinline__ int box_node(const TileBox& b, const Axis4& ax, const Axis4& az, int i, int j) {
    return (ax.base + i - b.X0) * b.NZ + (az.base + j - b.Z0);
}

// km_g2p_tile: G2P (n2p.jl:14-40, tplgy.jl:43-62) fused with the mUSL momentum P2G (augm.jl:13-25)
// in the tile form of km_p2g_tile.  A CTA owns TC consecutive cells and stages their stencil data
// and the (v, a) box of the grid update; each thread takes one list slot of the cells' slice at a
// time (the point's PIC/FLIP update, new position and cell, vmax and next-cell counts exactly as
// g2p_seg_body), with the next slot's list entries already loading, and stages its weights and m v;
// then the four lanes of a cell add their stencil column's m v over the cell's points, as
// km_aux_tile<.., 1> does from the stored velocities, and one FP32 atomic per node and component
// reaches the grid.  Standard and TPIC transfers (APIC's Bᵢⱼ pass and the deterministic mode keep
// km_g2p_seg).
// SOLVE: the grid update runs here instead of in km_solve: the box is staged as the P2G's m, p, f
// and Dirichlet word of each node (cp.async, in the space the point staging uses afterwards) and
// turned into (v, a) by grid_update; every tile's box must then fit TB_SOLVE nodes (the host checks).
constexpr int TG_STRIDE = 11;   // floats per staged point: wx[4], wz[4], m vx, m vz (odd: no bank conflicts)
constexpr int TB_SOLVE = 832;

template <int BASIS, int TC, bool SOLVE = false>
__global__ void __launch_bounds__(4 * TC) km_g2p_tile(MCtx A) {
    constexpr int NT = 4 * TC;
    constexpr int NB = SOLVE ? TB_SOLVE : TB_MAX;
    constexpr int NSP = NT * TG_STRIDE, NRAW = SOLVE ? 6 * TB_SOLVE : 0;
    __shared__ __align__(16) float sp[NSP > NRAW ? NSP : NRAW];
    __shared__ __align__(16) float4 box[NB];
    __shared__ int4 cinfo[TC];
    const int c0 = blockIdx.x * TC;
    if (c0 >= A.g.ncell) return;
    const int c1 = min(c0 + TC, A.g.ncell);
    // the tile's stencil data depend on the mesh only: staged before the wait for the previous kernel
    stage_cells(A.g, c0, c1, cinfo);
    pdl_enter();
    EP_ACTIVE(A.ctl);
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int* start = A.S.start[cur];
    const int b0 = start[c0], b1 = start[c1];
    if (SOLVE && A.cf.locking) {
        // the F-bar pass adds Σ N m δJ into z of the packed node values and km_cons scales it by w:
        // z = 0 and w = 1/m of the nodes this tile owns (node (ex, ez) of each cell, and the last
        // node row / column with the last cells), empty tiles included
        float2* zw = reinterpret_cast<float2*>(A.N.vg4) + 1;
        for (int i = threadIdx.x; i < c1 - c0; i += NT) {
            const int c = c0 + i, ex = c / A.g.nel[1], ez = c - ex * A.g.nel[1];
            const int lx = ex == A.g.nel[0] - 1, lz = ez == A.g.nel[1] - 1;
            for (int ox = 0; ox <= lx; ++ox)
                for (int oz = 0; oz <= lz; ++oz) {
                    const size_t n = (size_t)(ez + oz) + (size_t)A.g.nno[1] * (ex + ox);
                    const float m = A.N.m[n];
                    zw[2 * n] = make_float2(0.f, m != 0.f ? 1.f / m : 0.f);
                }
        }
    }
    if (b0 == b1) return;
    const int t = threadIdx.x, lane = t & 31;
    const int q = t & 3, cl = c0 + (t >> 2);
    const bool cell_ok = cl < c1;
    // the first slot's list entries, then the tile's stencil data and node box
    int p_n = -1, c_n = -1;
    if (b0 + t < b1) {
        p_n = A.S.list[cur][b0 + t];
        c_n = A.S.cellof[cur][b0 + t];
    }
    const int pb = cell_ok ? start[cl] : 0, pe = cell_ok ? start[cl + 1] : 0;
    int NX;
    const TileBox tb = tile_box(A.g, c0, c1, NX, NB);
    if (SOLVE && !tb.staged) {            // the host launches SOLVE only when every box fits
        if (t == 0) set_err(A.ctl, EP_ERR_ARG, c0);
        return;
    }
    const int nbox = NX * tb.NZ;
    const float dtf = (float)A.ctl->dt, Cpf = (float)A.cf.Cpf;
    if (SOLVE) {
        // the P2G fields of the box nodes: raw[q * NB + i], q = m, p_x, p_z, f_x, f_z, Dirichlet word
        float* raw = sp;
        const float* fld[5] = {A.N.m, A.N.p[0], A.N.p[1], A.N.f[0], A.N.f[1]};
        for (int i = t; i < nbox; i += NT) {
            int bx = 0, bz = i;
            while (bz >= tb.NZ) {
                bz -= tb.NZ;
                ++bx;
            }
            const int nx = tb.X0 + bx, nz = tb.Z0 + bz;
            const bool ok = nx >= 0 && nx < A.g.nno[0] && nz >= 0 && nz < A.g.nno[1];
            const size_t n = ok ? (size_t)nz + (size_t)A.g.nno[1] * nx : 0;
#pragma unroll
            for (int f = 0; f < 5; ++f) cp_async_zfill<4>(raw + f * NB + i, fld[f] + n, ok);
            cp_async_zfill<4>(raw + 5 * NB + i, A.g.bcw + n, ok);
        }
    } else if (tb.staged) {
        stage_box(A.g, A.N.va4, box, tb, NX);
    }
    const float4* vb = (SOLVE || tb.staged) ? box : A.N.va4;
    const float hx = (float)A.g.h[0], hz = (float)A.g.h[1];
    const float ihx = 1.f / hx, ihz = 1.f / hz;
    float acc[4][2];
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j][0] = acc[j][1] = 0.f;
    unsigned vm0 = 0u, vm1 = 0u;
    bool bad = false;
    cp_async_wait_all();
    __syncthreads();
    if (SOLVE) {
        const float eta = (float)A.cf.damping;
        for (int i = t; i < nbox; i += NT) {
            const float* raw = sp + i;
            const float pn[2] = {raw[NB], raw[2 * NB]};
            float f[3] = {raw[3 * NB], raw[4 * NB], 0.f}, a[3], v[3];
            grid_update(2, raw[0], pn, f, __float_as_int(raw[5 * NB]), dtf, eta, a, v);
            box[i] = make_float4(v[0], v[1], a[0], a[1]);
        }
        __syncthreads();      // sp now stages points
    }
    for (int ch = b0; ch < b1; ch += NT) {
        const int k = ch + t;
        const int p = p_n, c = c_n;
        p_n = c_n = -1;
        if (k + NT < b1) {
            p_n = A.S.list[cur][k + NT];
            c_n = A.S.cellof[cur][k + NT];
        }
        int c2 = -1;
        if (k < b1) {
            Axis4 ax, az;
            const int4 ci = cinfo[c - c0];
            cell_axes(ci, ax, az);
            const int ex = ci.x, ez = ci.y;
            const float dx = A.P.dx[cur][0][p], dz = A.P.dx[cur][1][p];
            const float lx = BASIS == EP_BASIS_GIMPM ? A.P.l[0][p] : 0.f;
            const float lz = BASIS == EP_BASIS_GIMPM ? A.P.l[1][p] : 0.f;
            float wx[4], dwx[4], wz[4], dwz[4];
            axis_w<BASIS>(ax, dx, hx, ihx, lx, wx, dwx, bad);
            axis_w<BASIS>(az, dz, hz, ihz, lz, wz, dwz, bad);
            float vpx = 0.f, vpz = 0.f, afx = 0.f, afz = 0.f;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (ax.cls[i] < 0) continue;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (az.cls[j] < 0) continue;
                    const float N = wx[i] * wz[j];
                    const float4 nv = vb[box_node(tb, ax, az, i, j)];
                    vpx += N * nv.x;
                    vpz += N * nv.y;
                    afx += N * nv.z;
                    afz += N * nv.w;
                }
            }
            const float vx = Cpf * (A.P.v[0][p] + dtf * afx) + (1.f - Cpf) * vpx;
            const float vz = Cpf * (A.P.v[1][p] + dtf * afz) + (1.f - Cpf) * vpz;
            A.P.v[0][p] = vx;
            A.P.v[1][p] = vz;
            vm0 = max(vm0, __float_as_uint(fabsf(vx)));
            vm1 = max(vm1, __float_as_uint(fabsf(vz)));
            const float ox = dx + dtf * vpx, oz = dz + dtf * vpz;
            if (isfinite(ox) && isfinite(oz)) {
                int ex2, ez2;
                float o2x, o2z;
                recell(A.g, 0, ex, ox, ihx, ex2, o2x);
                recell(A.g, 1, ez, oz, ihz, ez2, o2z);
                c2 = ez2 + A.g.nel[1] * ex2;
                A.P.dx[nxt][0][p] = o2x;
                A.P.dx[nxt][1][p] = o2z;
            } else {
                set_err(A.ctl, EP_ERR_NONFINITE, p);
            }
            A.P.p2e_next[p] = c2;
            if (A.P.pcell[nxt]) A.P.pcell[nxt][p] = c2;
            const float mp = A.P.mp[p];
            float* st = sp + t * TG_STRIDE;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                st[i] = ax.cls[i] < 0 ? 0.f : wx[i];
                st[4 + i] = az.cls[i] < 0 ? 0.f : wz[i];
            }
            st[8] = mp * vx;
            st[9] = mp * vz;
        }
        {
            // next-cell counts: one atomic per distinct cell of the warp
            const unsigned mm = __match_any_sync(0xffffffffu, c2);
            if (c2 >= 0 && lane == __ffs(mm) - 1) atomicAdd(&A.S.count[nxt][c2], __popc(mm));
        }
        __syncthreads();
        // this lane's cell: the mUSL momentum of its stencil column over the cell's points in the chunk
        const int lo = max(pb, ch), hi = min(pe, min(ch + NT, b1));
        for (int kk = lo; kk < hi; ++kk) {
            const float* st = sp + (kk - ch) * TG_STRIDE;
            const float wq = st[q];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float N = wq * st[4 + j];
                acc[j][0] += N * st[8];
                acc[j][1] += N * st[9];
            }
        }
        __syncthreads();
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, c0);
    // vmax over the warp, one atomic per warp (non-negative floats order like their bits)
    vm0 = __reduce_max_sync(0xffffffffu, vm0);
    vm1 = __reduce_max_sync(0xffffffffu, vm1);
    if (lane == 0) {
        if (vm0) atomicMax(&A.ctl->vmax_bits[0], (unsigned long long)__double_as_longlong((double)__uint_as_float(vm0)));
        if (vm1) atomicMax(&A.ctl->vmax_bits[1], (unsigned long long)__double_as_longlong((double)__uint_as_float(vm1)));
    }
    if (!cell_ok || pb == pe) return;
    Axis4 ax, az;
    cell_axes(cinfo[cl - c0], ax, az);
    if (ax.cls[q] < 0) return;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (az.cls[j] < 0) continue;
        const int n = node2(A.g, ax, az, q, j);
        atomicAdd(&A.N.pm[0][n], acc[j][0]);
        atomicAdd(&A.N.pm[1][n], acc[j][1]);
    }
}


// km_p2g_tile: m, p, f (p2n.jl:135-155 std, 217-240 tpic).  A CTA owns TP_CELLS
// (16, 32 or 64: the tile shape the autotuner picks) consecutive cells, whose
// points form one slice of the sorted list.  The slice
// is staged through shared memory in chunks of one point per thread (point data
// and shape values computed once per point), then four lanes per cell -- lane q
// owns stencil column q -- accumulate the column's 4 nodes x 5 quantities in
// registers over the cell's staged points, and add them to the grid with one
// FP32 atomic per node and quantity.
constexpr int TP_STRIDE = 29;   // floats per staged point (odd: no bank conflicts)

// NT: threads of the block (the staging width); 4 TP_CELLS of them accumulate, the rest only stage
// EARLY (the stand-alone kernel, a programmatic dependent launch): the tile's stencil data, which depend
// on the mesh only, are staged before the wait for the previous kernel of the stream
template <int BASIS, int TP_CELLS, bool DET, int NT = 4 * TP_CELLS, bool EARLY = false>
__device__ __forceinline__ void p2g_tile_body(const MCtx& A, int bid) {
    static_assert(NT >= 4 * TP_CELLS, "a P2G tile needs 4 lanes per cell");
    constexpr int TP_THREADS = NT;
    if (blockDim.x != NT) {                  // launch shape and body disagree: report, touch nothing
        if (threadIdx.x == 0) set_err(A.ctl, EP_ERR_ARG, -1);
        return;
    }
    __shared__ float sp[TP_THREADS * TP_STRIDE];
    __shared__ int4 cinfo[TP_CELLS];
    if (EARLY) {
        if (bid * TP_CELLS >= A.g.ncell) return;
        stage_cells(A.g, bid * TP_CELLS, min(bid * TP_CELLS + TP_CELLS, A.g.ncell), cinfo);
        pdl_enter();
    }
    EP_ACTIVE(A.ctl);
    const int cur = A.ctl->parity;
    const int c0 = bid * TP_CELLS;
    if (c0 >= A.g.ncell) return;
    const int c1 = min(c0 + TP_CELLS, A.g.ncell);
    const int* start = A.S.start[cur];
    const int b0 = start[c0], b1 = start[c1];
    if (b0 == b1) return;
    const int t = threadIdx.x;
    const int q = t & 3, cl = c0 + (t >> 2);          // this lane's cell and stencil column
    const bool cell_ok = cl < c1;
    // the first slot's list entries, then the tile's stencil data (as km_g2p_tile)
    int p_n = -1, c_n = -1;
    if (b0 + t < b1) {
        p_n = A.S.list[cur][b0 + t];
        c_n = A.S.cellof[cur][b0 + t];
    }
    const int pb = cell_ok ? start[cl] : 0, pe = cell_ok ? start[cl + 1] : 0;
    if (!EARLY) {
        __syncthreads();      // a persistent caller's previous tile may still read cinfo
        stage_cells(A.g, c0, c1, cinfo);
    }
    const float hx = (float)A.g.h[0], hz = (float)A.g.h[1];
    const float gz = (float)A.ctl->g[1];
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    const bool tpic = A.cf.trsfr != EP_TRSFR_STD;   // v + G δ: TPIC's ∇v or APIC's Bᵢⱼ (D⁻¹ = I) in dv
    float am[4], apx[4], apz[4], afx[4], afz[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) am[j] = apx[j] = apz[j] = afx[j] = afz[j] = 0.f;
    bool bad = false;
    __syncthreads();
    for (int ch = b0; ch < b1; ch += TP_THREADS) {
        // stage one point per thread
        const int k = ch + t;
        const int p = p_n, c = c_n;
        p_n = c_n = -1;
        if (k + TP_THREADS < b1) {
            p_n = A.S.list[cur][k + TP_THREADS];
            c_n = A.S.cellof[cur][k + TP_THREADS];
        }
        if (k < b1) {
            Axis4 ax, az;
            cell_axes(cinfo[c - c0], ax, az);
            const float dx = A.P.dx[cur][0][p], dz = A.P.dx[cur][1][p];
            const float lx = BASIS == EP_BASIS_GIMPM ? A.P.l[0][p] : 0.f;
            const float lz = BASIS == EP_BASIS_GIMPM ? A.P.l[1][p] : 0.f;
            float* s = sp + t * TP_STRIDE;
            axis_w<BASIS>(ax, dx, hx, 1.f / hx, lx, s + 0, s + 4, bad);      // wx, dwx
            axis_w<BASIS>(az, dz, hz, 1.f / hz, lz, s + 8, s + 12, bad);     // wz, dwz
            const float sc = fin ? A.P.Om0[p] : A.P.Om[p];                  // Ω σ = Ω0 τ (finite) or Ω σ
            s[16] = A.P.mp[p];
            s[17] = A.P.v[0][p];
            s[18] = A.P.v[1][p];
            s[19] = sc * A.P.tau[0][p];
            s[20] = sc * A.P.tau[1][p];
            s[21] = sc * A.P.tau[2][p];
            if (tpic) {
                s[22] = dx;
                s[23] = dz;
                s[24] = A.P.dv[0][p];
                s[25] = A.P.dv[1][p];
                s[26] = A.P.dv[2][p];
                s[27] = A.P.dv[3][p];
            }
        }
        __syncthreads();
        // this lane's cell: its points inside the chunk
        const int lo = max(pb, ch), hi = min(pe, min(ch + TP_THREADS, b1));
        for (int kk = lo; kk < hi; ++kk) {
            const float* s = sp + (kk - ch) * TP_STRIDE;
            const float wq = s[q], dwq = s[4 + q];
            const float ms = s[16], vx = s[17], vz = s[18], txx = s[19], tzz = s[20], txz = s[21];
            float vxi = vx, vzi = vz, gxz = 0.f, gzz = 0.f, dzp = 0.f;
            if (tpic) {
                // v + ∇v (x_n - x_p) with the previous step's ∇v (p2n.jl:233-235)
                const float ddx = (float)(q - 1) * hx - s[22];
                dzp = s[23];
                vxi = vx + s[24] * ddx;
                vzi = vz + s[25] * ddx;
                gxz = s[26];
                gzz = s[27];
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float wz = s[8 + j], dwz = s[12 + j];
                const float N = wq * wz, Nx = dwq * wz, Nz = wq * dwz;
                const float Nm = N * ms;
                am[j] += Nm;
                if (!tpic) {
                    apx[j] += Nm * vx;
                    apz[j] += Nm * vz;
                } else {
                    const float ddz = (float)(j - 1) * hz - dzp;
                    apx[j] += Nm * (vxi + gxz * ddz);
                    apz[j] += Nm * (vzi + gzz * ddz);
                }
                afx[j] -= Nx * txx + Nz * txz;
                afz[j] -= (Nx * txz + Nz * tzz) - Nm * gz;
            }
        }
        __syncthreads();
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, c0);
    if (!cell_ok || pb == pe) return;
    if (DET) {
        // the cell's partial sums, node (q, j) of its stencil; km_gather adds them in a fixed order
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float* o = A.part + ((size_t)cl * 16 + q * 4 + j) * 5;
            o[0] = am[j]; o[1] = apx[j]; o[2] = apz[j]; o[3] = afx[j]; o[4] = afz[j];
        }
        return;
    }
    Axis4 ax, az;
    cell_axes(cinfo[cl - c0], ax, az);
    if (ax.cls[q] < 0) return;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (az.cls[j] < 0) continue;
        const int n = node2(A.g, ax, az, q, j);
        atomicAdd(&A.N.m[n], am[j]);
        atomicAdd(&A.N.p[0][n], apx[j]);
        atomicAdd(&A.N.p[1][n], apz[j]);
        atomicAdd(&A.N.f[0][n], afx[j]);
        atomicAdd(&A.N.f[1][n], afz[j]);
    }
}

template <int BASIS, int TP_CELLS, bool DET>
__global__ void __launch_bounds__(4 * TP_CELLS) km_p2g_tile(MCtx A) {
    p2g_tile_body<BASIS, TP_CELLS, DET, 4 * TP_CELLS, true>(A, blockIdx.x);
}


// Deterministic scatters of the mUSL momentum (KIND 1: m v per point, augm.jl:13-25) and of
// Σ N m δJ (KIND 2: the per-point value left in ptmp by km_fbar_seg, volumetric.jl:1-11): the
// tile staging of km_p2g_tile, each cell's points summed in list (point id) order into the
// cell's node partials.
// ATOMIC: the cell sums go to the nodes with FP32 atomics (else per-cell partials for km_gather)
template <int BASIS, int TP_CELLS, int KIND, bool ATOMIC = false>
__global__ void __launch_bounds__(4 * TP_CELLS) km_aux_tile(MCtx A) {
    constexpr int TP_THREADS = 4 * TP_CELLS, NQ = KIND == 1 ? 2 : 1, ST = 11;
    EP_ACTIVE(A.ctl);
    __shared__ float sp[TP_THREADS * ST];
    const int cur = A.ctl->parity;
    const int c0 = blockIdx.x * TP_CELLS;
    if (c0 >= A.g.ncell) return;
    const int c1 = min(c0 + TP_CELLS, A.g.ncell);
    const int* start = A.S.start[cur];
    const int b0 = start[c0], b1 = start[c1];
    if (b0 == b1) return;
    const int t = threadIdx.x;
    const int q = t & 3, cl = c0 + (t >> 2);
    const bool cell_ok = cl < c1;
    const int pb = cell_ok ? start[cl] : 0, pe = cell_ok ? start[cl + 1] : 0;
    const float hx = (float)A.g.h[0], hz = (float)A.g.h[1];
    float acc[4][NQ];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int v = 0; v < NQ; ++v) acc[j][v] = 0.f;
    bool bad = false;
    for (int ch = b0; ch < b1; ch += TP_THREADS) {
        const int k = ch + t;
        if (k < b1) {
            const int p = A.S.list[cur][k], c = A.S.cellof[cur][k];
            const int ex = c / A.g.nel[1], ez = c - ex * A.g.nel[1];
            const Axis4 ax = axis4(A.g, 0, ex), az = axis4(A.g, 1, ez);
            const float lx = BASIS == EP_BASIS_GIMPM ? A.P.l[0][p] : 0.f;
            const float lz = BASIS == EP_BASIS_GIMPM ? A.P.l[1][p] : 0.f;
            float* s = sp + t * ST;
            float dw[4];
            axis_w<BASIS>(ax, A.P.dx[cur][0][p], hx, 1.f / hx, lx, s + 0, dw, bad);
            axis_w<BASIS>(az, A.P.dx[cur][1][p], hz, 1.f / hz, lz, s + 4, dw, bad);
            if (KIND == 1) {
                const float mp = A.P.mp[p];
                s[8] = mp * A.P.v[0][p];
                s[9] = mp * A.P.v[1][p];
            } else {
                s[8] = A.ptmp[p];
            }
        }
        __syncthreads();
        const int lo = max(pb, ch), hi = min(pe, min(ch + TP_THREADS, b1));
        for (int kk = lo; kk < hi; ++kk) {
            const float* s = sp + (kk - ch) * ST;
            const float wq = s[q];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float N = wq * s[4 + j];
#pragma unroll
                for (int v = 0; v < NQ; ++v) acc[j][v] += N * s[8 + v];
            }
        }
        __syncthreads();
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, c0);
    if (!cell_ok || pb == pe) return;
    if (ATOMIC) {
        const int ex = cl / A.g.nel[1], ez = cl - ex * A.g.nel[1];
        const Axis4 ax = axis4(A.g, 0, ex), az = axis4(A.g, 1, ez);
        if (ax.cls[q] < 0) return;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (az.cls[j] < 0) continue;
            const int n = node2(A.g, ax, az, q, j);
            if (KIND == 1) {
                atomicAdd(&A.N.pm[0][n], acc[j][0]);
                atomicAdd(&A.N.pm[1][n], acc[j][NQ - 1]);
            } else {
                atomicAdd(&A.N.dJacc[n], acc[j][0]);
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int v = 0; v < NQ; ++v) A.part[((size_t)cl * 16 + q * 4 + j) * NQ + v] = acc[j][v];
    }
}

// node sums of the per-cell partials: the cells whose stencil holds node (ix, jz) are
// ex = ix + 1 - q, ez = jz + 1 - r (q, r = 0..3), visited in that fixed order
template <int NQ>
__global__ void km_gather(MCtx A, float* o0, float* o1, float* o2, float* o3, float* o4) {
    EP_ACTIVE(A.ctl);
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= A.g.nnode) return;
    const int cur = A.ctl->parity;
    const int nz = A.g.nno[1], ix = n / nz, jz = n - ix * nz;
    const int* start = A.S.start[cur];
    float acc[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) acc[v] = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ex = ix + 1 - q;
        if (ex < 0 || ex >= A.g.nel[0]) continue;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int ez = jz + 1 - r;
            if (ez < 0 || ez >= A.g.nel[1]) continue;
            const int c = ez + A.g.nel[1] * ex;
            if (start[c] == start[c + 1]) continue;
            const float* pp = A.part + ((size_t)c * 16 + q * 4 + r) * NQ;
#pragma unroll
            for (int v = 0; v < NQ; ++v) acc[v] += pp[v];
        }
    }
    float* outs[5] = {o0, o1, o2, o3, o4};
#pragma unroll
    for (int v = 0; v < NQ; ++v) outs[v][n] = acc[v];
}

// point ids of each cell's list segment in ascending order (deterministic summation order)
__global__ void km_sort_cells(MCtx A, int which) {
    if (which == 0 && !A.ctl->active) return;
    const int par = which == 0 ? (A.ctl->parity ^ 1) : A.ctl->parity;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.g.ncell) return;
    int* L = A.S.list[par];
    const int b = A.S.start[par][c], e = A.S.start[par][c + 1];
    for (int i = b + 1; i < e; ++i) {
        const int v = L[i];
        int j = i - 1;
        while (j >= b && L[j] > v) {
            L[j + 1] = L[j];
            --j;
        }
        L[j + 1] = v;
    }
}

// km_vmusl: mUSL nodal velocity v = p/m with Dirichlet masks (augm.jl:37-53)
__device__ __forceinline__ void vmusl_one(const MCtx& A, int n) {
    const float m = A.N.m[n];
    const float mi = m != 0.f ? 1.f / m : 0.f;
    float vv[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < A.g.dim; ++d) {
        float v = 0.f;
        if (m != 0.f && !A.g.bcs[(size_t)d * A.g.nnode + n]) v = A.N.pm[d][n] * mi;
        A.N.vm[d][n] = v;
        vv[d] = v;
    }
    if (A.g.dim == 2) A.N.vg4[n] = make_float4(vv[0], vv[1], 0.f, mi);
}

__device__ __forceinline__ void vmusl_body(const MCtx& A, int bid) {
    EP_ACTIVE(A.ctl);
    const int n = bid * blockDim.x + threadIdx.x;
    if (n < A.g.nnode) vmusl_one(A, n);
}

__global__ void km_vmusl(MCtx A) { vmusl_body(A, blockIdx.x); }


__device__ __forceinline__ void place_next(const MCtx& A, int p, int nxt) {
    const int c2 = A.P.p2e_next[p];
    if (c2 < 0) return;
    const int k = atomicAdd(&A.S.cursor[c2], 1);
    const int pos = A.S.start[nxt][c2] + k;
    if (pos < A.S.start[nxt][c2 + 1]) {
        A.S.list[nxt][pos] = p;
        A.S.cellof[nxt][pos] = c2;
    } else {
        set_err(A.ctl, EP_ERR_CUDA, p);
    }
}

// place_next for a whole warp: one cursor atomic per distinct cell (c2 < 0: nothing to place)
__device__ __forceinline__ void place_next_warp(const MCtx& A, int p, int c2, int nxt, int lane) {
    const unsigned mm = __match_any_sync(0xffffffffu, c2);
    const int leader = __ffs(mm) - 1;
    int base = 0;
    if (lane == leader && c2 >= 0) base = atomicAdd(&A.S.cursor[c2], __popc(mm));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (c2 < 0) return;
    const int pos = A.S.start[nxt][c2] + base + __popc(mm & ((1u << lane) - 1u));
    if (pos < A.S.start[nxt][c2 + 1]) {
        A.S.list[nxt][pos] = p;
        A.S.cellof[nxt][pos] = c2;
    } else {
        set_err(A.ctl, EP_ERR_CUDA, p);
    }
}

// km_fbar_seg: δJ = det(I + dt ∇v) - 1 and its P2G Σ N m δJ (deform.jl:9-18,
// volumetric.jl:1-11), one lane per point; places the points into the next lists
template <int BASIS, bool DET>
__device__ __forceinline__ void fbar_seg_body(const MCtx& A, int bid) {
    EP_ACTIVE(A.ctl);
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int n = A.S.start[cur][A.g.ncell];
    const int k = bid * blockDim.x + threadIdx.x;
    bool bad = false;
    PtW W;
    const bool live = point_of<BASIS>(A, cur, k, n, W, bad);
    const Seg S = seg_of(W.c);
    const float dtf = (float)A.ctl->dt;
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    float mdj = 0.f;
    if (live) {
        float g00 = 0.f, g01 = 0.f, g10 = 0.f, g11 = 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (W.ax.cls[i] < 0) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (W.az.cls[j] < 0) continue;
                const int nd = node2(A.g, W.ax, W.az, i, j);
                const float Nx = W.dwx[i] * W.wz[j], Nz = W.wx[i] * W.dwz[j];
                const float2 q = *reinterpret_cast<const float2*>(&A.N.vg4[nd]);
                const float vx = q.x, vz = q.y;
                g00 += Nx * vx;
                g01 += Nz * vx;
                g10 += Nx * vz;
                g11 += Nz * vz;
            }
        }
        A.P.gv[k] = make_float4(g00, g10, g01, g11);   // km_cons reads the slot's ∇v back
        const float D00 = dtf * g00, D10 = dtf * g10, D01 = dtf * g01, D11 = dtf * g11;
        const float dJ = D00 + D11 + (D00 * D11 - D01 * D10);
        // numerator mass ρΩ after the deformation update: finite ρ0Ω0 (unchanged), infinitesimal
        // ρ J Ω0 = m (1 + δJ), so the nodal sum carries m (1+δJ)^2 - m = m δJ (2 + δJ) (volumetric.jl:8)
        mdj = A.P.mp[W.p] * (fin ? dJ : dJ * (2.f + dJ));
    }
    place_next_warp(A, live ? W.p : -1, live ? A.P.p2e_next[W.p] : -1, nxt, S.lane);
    if (DET) {
        if (live) A.ptmp[W.p] = mdj;             // km_aux_tile<.., 2> scatters it
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float v = seg_sum(live ? W.wx[i] * W.wz[j] * mdj : 0.f, S);
                if (S.head && live && W.ax.cls[i] >= 0 && W.az.cls[j] >= 0)
                    atomicAdd(&A.N.dJacc[node2(A.g, W.ax, W.az, i, j)], v);
            }
        }
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, W.c);
}

template <int BASIS, bool DET>
__global__ void __launch_bounds__(256) km_fbar_seg(MCtx A) {
    fbar_seg_body<BASIS, DET>(A, blockIdx.x);
}


// km_fbar_tile: km_fbar_seg in the tile form of km_p2g_tile, with the tile's stencil data and the
// velocity box staged as in km_g2p_tile.  Each thread takes one list slot of the CTA's cells at a time
// (∇v, δJ and m δJ exactly as fbar_seg_body, and the point's place in the next lists), stages its
// weights and m δJ, and the four lanes of a cell add Σ N m δJ over the cell's points for their
// stencil column: one FP32 atomic per node and cell instead of segmented warp sums over the 16
// nodes of every point.
// VM: the mUSL nodal velocity (augm.jl:37-53, vmusl_one) is formed here from the staged m, mUSL p and
// Dirichlet word of the box nodes instead of in km_vmusl_scan (the boxes fit TB_SOLVE nodes).
constexpr int TF_STRIDE = 9;    // floats per staged point: wx[4], wz[4], m δJ (odd: no bank conflicts)

template <int BASIS, int TC, bool VM = false>
__global__ void __launch_bounds__(4 * TC) km_fbar_tile(MCtx A) {
    constexpr int NT = 4 * TC;
    constexpr int NB = VM ? TB_SOLVE : TB_MAX;
    constexpr int NSP = NT * TF_STRIDE, NRAW = VM ? 4 * TB_SOLVE : 0;
    __shared__ __align__(16) float sp[NSP > NRAW ? NSP : NRAW];
    __shared__ __align__(16) float2 box[NB];
    __shared__ int4 cinfo[TC];
    const int c0 = blockIdx.x * TC;
    if (c0 >= A.g.ncell) return;
    const int c1 = min(c0 + TC, A.g.ncell);
    // the tile's stencil data depend on the mesh only: staged before the wait for the previous kernel
    stage_cells(A.g, c0, c1, cinfo);
    pdl_enter();
    EP_ACTIVE(A.ctl);
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int* start = A.S.start[cur];
    const int b0 = start[c0], b1 = start[c1];
    if (b0 == b1) return;
    const int t = threadIdx.x, lane = t & 31;
    const int q = t & 3, cl = c0 + (t >> 2);
    const bool cell_ok = cl < c1;
    int p_n = -1, c_n = -1;
    if (b0 + t < b1) {
        p_n = A.S.list[cur][b0 + t];
        c_n = A.S.cellof[cur][b0 + t];
    }
    const int pb = cell_ok ? start[cl] : 0, pe = cell_ok ? start[cl + 1] : 0;
    int NX;
    const TileBox tb = tile_box(A.g, c0, c1, NX, NB);
    if (VM && !tb.staged) {               // the host launches VM only when every box fits
        if (t == 0) set_err(A.ctl, EP_ERR_ARG, c0);
        return;
    }
    const int nbox = NX * tb.NZ;
    if (VM) {
        // raw[q * NB + i], q = m, mUSL p_x, mUSL p_z, Dirichlet word
        float* raw = sp;
        const float* fld[3] = {A.N.m, A.N.pm[0], A.N.pm[1]};
        for (int i = t; i < nbox; i += NT) {
            int bx = 0, bz = i;
            while (bz >= tb.NZ) {
                bz -= tb.NZ;
                ++bx;
            }
            const int nx = tb.X0 + bx, nz = tb.Z0 + bz;
            const bool ok = nx >= 0 && nx < A.g.nno[0] && nz >= 0 && nz < A.g.nno[1];
            const size_t n = ok ? (size_t)nz + (size_t)A.g.nno[1] * nx : 0;
#pragma unroll
            for (int f = 0; f < 3; ++f) cp_async_zfill<4>(raw + f * NB + i, fld[f] + n, ok);
            cp_async_zfill<4>(raw + 3 * NB + i, A.g.bcw + n, ok);
        }
    } else if (tb.staged) {
        stage_box(A.g, A.N.vg4, box, tb, NX);
    }
    const float hx = (float)A.g.h[0], hz = (float)A.g.h[1];
    const float dtf = (float)A.ctl->dt;
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    bool bad = false;
    cp_async_wait_all();
    __syncthreads();
    if (VM) {
        for (int i = t; i < nbox; i += NT) {
            const float m = sp[i];
            const int bc = __float_as_int(sp[3 * NB + i]);
            const float mi = m != 0.f ? 1.f / m : 0.f;
            const float vx = (m != 0.f && !(bc & 1)) ? sp[NB + i] * mi : 0.f;
            const float vz = (m != 0.f && !(bc & 2)) ? sp[2 * NB + i] * mi : 0.f;
            box[i] = make_float2(vx, vz);
        }
        __syncthreads();      // sp now stages points
    }
    for (int ch = b0; ch < b1; ch += NT) {
        const int k = ch + t;
        const int p = p_n, c = c_n;
        p_n = c_n = -1;
        if (k + NT < b1) {
            p_n = A.S.list[cur][k + NT];
            c_n = A.S.cellof[cur][k + NT];
        }
        int c2 = -1;
        if (k < b1) {
            Axis4 ax, az;
            cell_axes(cinfo[c - c0], ax, az);
            const float lx = BASIS == EP_BASIS_GIMPM ? A.P.l[0][p] : 0.f;
            const float lz = BASIS == EP_BASIS_GIMPM ? A.P.l[1][p] : 0.f;
            float wx[4], dwx[4], wz[4], dwz[4];
            axis_w<BASIS>(ax, A.P.dx[cur][0][p], hx, 1.f / hx, lx, wx, dwx, bad);
            axis_w<BASIS>(az, A.P.dx[cur][1][p], hz, 1.f / hz, lz, wz, dwz, bad);
            float g00 = 0.f, g01 = 0.f, g10 = 0.f, g11 = 0.f;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (ax.cls[i] < 0) continue;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (az.cls[j] < 0) continue;
                    const float Nx = dwx[i] * wz[j], Nz = wx[i] * dwz[j];
                    const float2 vn = (VM || tb.staged)
                                          ? box[box_node(tb, ax, az, i, j)]
                                          : *reinterpret_cast<const float2*>(&A.N.vg4[node2(A.g, ax, az, i, j)]);
                    g00 += Nx * vn.x;
                    g01 += Nz * vn.x;
                    g10 += Nx * vn.y;
                    g11 += Nz * vn.y;
                }
            }
            A.P.gv[k] = make_float4(g00, g10, g01, g11);
            const float D00 = dtf * g00, D10 = dtf * g10, D01 = dtf * g01, D11 = dtf * g11;
            const float dJ = D00 + D11 + (D00 * D11 - D01 * D10);
            // the numerator mass after the deformation update, as fbar_seg_body (volumetric.jl:8)
            const float mdj = A.P.mp[p] * (fin ? dJ : dJ * (2.f + dJ));
            float* st = sp + t * TF_STRIDE;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                st[i] = ax.cls[i] < 0 ? 0.f : wx[i];
                st[4 + i] = az.cls[i] < 0 ? 0.f : wz[i];
            }
            st[8] = mdj;
            c2 = A.P.p2e_next[p];
        }
        place_next_warp(A, k < b1 ? p : -1, c2, nxt, lane);
        __syncthreads();
        const int lo = max(pb, ch), hi = min(pe, min(ch + NT, b1));
        for (int kk = lo; kk < hi; ++kk) {
            const float* st = sp + (kk - ch) * TF_STRIDE;
            const float wq = st[q] * st[8];
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[j] += wq * st[4 + j];
        }
        __syncthreads();
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, c0);
    if (!cell_ok || pb == pe) return;
    Axis4 ax, az;
    cell_axes(cinfo[cl - c0], ax, az);
    if (ax.cls[q] < 0) return;
    // Σ N m δJ goes straight into the z slot of the packed node values, whose w holds 1/m: km_cons
    // takes the nodal δJ as z·w (no separate node pass)
    float* vz = reinterpret_cast<float*>(A.N.vg4) + 2;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (az.cls[j] >= 0) atomicAdd(vz + 4 * (size_t)node2(A.g, ax, az, q, j), acc[j]);
}


// km_dJn: nodal δJ_n = Σ N m δJ / m_n (volumetric.jl:12-22, increment form)
__device__ __forceinline__ void dJn_body(const MCtx& A, int bid) {
    EP_ACTIVE(A.ctl);
    const int n = bid * blockDim.x + threadIdx.x;
    if (n >= A.g.nnode) return;
    const float m = A.N.m[n];
    const float dj = (m == 0.f) ? 0.f : A.N.dJacc[n] / m;
    A.N.dJn[n] = dj;
    if (A.g.dim == 2) {
        float* q = reinterpret_cast<float*>(A.N.vg4) + 4 * (size_t)n;
        q[2] = dj;
        q[3] = 1.f;
    }
}

__global__ void km_dJn(MCtx A) {
    pdl_enter();
    dJn_body(A, blockIdx.x);
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

// The MC (2d, MCRetMap.jl) and modified Cam-Clay (camC/camCmodRetMap.jl) returns of one point as FP64
// islands (ep_scalar.h, the FP64 step's code) on the FP32 trial stress tt[NS]: their absolute
// tolerances (1e-6 Pa, 1e-6 Pa²) lie below the resolution of an FP32 stress.  Returns the new
// ϵpII[1] and sets *yielded; writes ϵpV (Cam-Clay) and reports a non-converged MC return.  Kept out
// of line so that the DP and J2 paths of the constitutive kernels keep their registers.
template <int NS>
__device__ __noinline__ float cons_iterative(const MCtx& A, int p, float* tt, float ep2, bool* yielded) {
    double s[NS];
    for (int i = 0; i < NS; ++i) s[i] = (double)tt[i];
    double g = 0.0;
    int y;
    if (A.cf.cons == EP_CONS_MC) {
        y = mc_return(s, (double)ep2, (double)A.P.c0[p], (double)A.P.cr[p], (double)A.P.sphi[p], (double)A.P.cphi[p],
                      (double)A.Hp, A.Deld, A.DelLU, A.piv, &g);
        if (y < 0) set_err(A.ctl, EP_ERR_NONCONVERGED, p);
    } else {
        double ev = A.P.epv[p];
        y = camc_return<NS>(s, (double)ep2, &ev, A.Kd, A.Deld, &g);
        if (y > 0) A.P.epv[p] = ev;
    }
    *yielded = y > 0;
    if (y > 0)
        for (int i = 0; i < NS; ++i) tt[i] = (float)s[i];
    return (float)g;
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
    for (int it = 1; fabsf(f) > fmaxf(1.0e-9f, 2.0e-7f * kap) && it < 20; ++it) {
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

// ---------------------------------------------------------------------------
// accumulated state: FP64 (ACC = 0) or double-float hi + lo (ACC = 1)

// hi + lo += inc (Knuth two-sum, then renormalise); FP32 instructions only
__device__ __forceinline__ void df_add(float& hi, float& lo, float inc) {
    const float s = hi + inc;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (inc - bb) + lo;
    const float t = s + e;
    lo = e - (t - s);
    hi = t;
}

// hi + lo = 1 + dev exactly representable pair for a deviation dev from 1
__device__ __forceinline__ void df_one_plus(float dev, float& hi, float& lo) {
    hi = 1.f + dev;
    lo = dev - (hi - 1.f);
}

// b = exp(2ε), ε = (e11, e22, e12), spectral form (DP.jl:65-66), as deviations from 1:
// b_ii - 1 = (E - 1) + E (cosh 2s - 1 ± sinh(2s)/s ε_d), b_12 = E sinh(2s)/s e12
__device__ __forceinline__ void exp2eps_dev(float e11, float e22, float e12, float em_expm1, float E, float* dev) {
    const float ed = 0.5f * (e11 - e22);
    const float s2 = ed * ed + e12 * e12;
    float chm1, shs;   // cosh(2s) - 1, sinh(2s)/s
    if (s2 < 1.0e-4f) {
        chm1 = s2 * (2.f + s2 * (2.f / 3.f));
        shs = 2.f * (1.f + s2 * (2.f / 3.f + s2 * (2.f / 15.f)));
    } else {
        const float s = sqrtf(s2);
        chm1 = coshf(2.f * s) - 1.f;
        shs = sinhf(2.f * s) / s;
    }
    dev[0] = em_expm1 + E * (chm1 + shs * ed);
    dev[1] = em_expm1 + E * (chm1 - shs * ed);
    dev[2] = E * (shs * e12);
}

// b_e = exp(2 eps) of a returned log strain (DP.jl:63-66), into the point's accumulated storage
template <int ACC>
__device__ __forceinline__ void rebuild_b(const MCtx& A, int p, float e11, float e22, float e12) {
    const float em = 0.5f * (e11 + e22);
    float E, Em1;
    if (ACC == 0) {
        const double Ed = ep_exp(2.0 * (double)em);   // e^{2 e_m} in FP64
        E = (float)Ed;
        Em1 = (float)(Ed - 1.0);
    } else {
        Em1 = expm1f(2.f * em);
        E = 1.f + Em1;
    }
    float dev[3];
    exp2eps_dev(e11, e22, e12, Em1, E, dev);
    if (ACC == 0) {
        A.P.bd[0][p] = 1.0 + (double)dev[0];
        A.P.bd[1][p] = 1.0 + (double)dev[1];
        A.P.bd[2][p] = (double)dev[2];
    } else {
        float h, l;
        df_one_plus(dev[0], h, l);
        A.P.bh[0][p] = h; A.P.bl[0][p] = l;
        df_one_plus(dev[1], h, l);
        A.P.bh[1][p] = h; A.P.bl[1][p] = l;
        A.P.bh[2][p] = dev[2]; A.P.bl[2][p] = 0.f;
    }
}

template <int ACC>
__device__ __forceinline__ void add_ep1(const MCtx& A, int p, float inc) {
    if (ACC == 0) {
        A.P.ep1d[p] += (double)inc;
    } else {
        float h = A.P.ep1h[p], l = A.P.ep1l[p];
        df_add(h, l, inc);
        A.P.ep1h[p] = h;
        A.P.ep1l[p] = l;
    }
}

// one rotation zeroing a[P][Q] of the symmetric a, accumulated into the columns of v
template <int P, int Q>
__device__ __forceinline__ void jrot3f(float (&a)[3][3], float (&v)[3][3]) {
    constexpr int R = 3 - P - Q;
    const float apq = a[P][Q];
    if (apq == 0.f) return;
    const float th = (a[Q][Q] - a[P][P]) / (2.f * apq);
    const float t = fabsf(th) > 1.0e15f ? 0.5f / th : copysignf(1.f, th) / (fabsf(th) + sqrtf(1.f + th * th));
    const float c = 1.f / sqrtf(1.f + t * t), sn = t * c;
    a[P][P] -= t * apq;
    a[Q][Q] += t * apq;
    a[P][Q] = a[Q][P] = 0.f;
    const float arp = a[R][P], arq = a[R][Q];
    a[R][P] = a[P][R] = c * arp - sn * arq;
    a[R][Q] = a[Q][R] = sn * arp + c * arq;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float vp = v[i][P], vq = v[i][Q];
        v[i][P] = c * vp - sn * vq;
        v[i][Q] = sn * vp + c * vq;
    }
}

// eigenvalues (diagonal of a on return) and eigenvectors (columns of v) of a symmetric 3x3;
// sweeps stop once the off-diagonal sum is below 1e-8 of the matrix norm (the eigenvalue error
// it leaves is below that, Weyl)
__device__ __forceinline__ void eig3f(float (&a)[3][3], float (&v)[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) v[i][j] = i == j ? 1.f : 0.f;
    const float nrm = fabsf(a[0][0]) + fabsf(a[1][1]) + fabsf(a[2][2]) +
                      2.f * (fabsf(a[0][1]) + fabsf(a[0][2]) + fabsf(a[1][2]));
#pragma unroll 1
    for (int sw = 0; sw < 8; ++sw) {
        if (fabsf(a[0][1]) + fabsf(a[0][2]) + fabsf(a[1][2]) <= 1.0e-8f * nrm) break;
        jrot3f<0, 1>(a, v);
        jrot3f<0, 2>(a, v);
        jrot3f<1, 2>(a, v);
    }
}

// det(I + D) - 1 of a 3x3 increment, without cancellation: tr D + principal minors + det D
__device__ __forceinline__ float det1p_m1(const float* D) {
    const float m2 = (D[0] * D[4] - D[3] * D[1]) + (D[0] * D[8] - D[6] * D[2]) + (D[4] * D[8] - D[7] * D[5]);
    const float d3 = D[0] * (D[4] * D[8] - D[7] * D[5]) - D[3] * (D[1] * D[8] - D[7] * D[2]) +
                     D[6] * (D[1] * D[5] - D[4] * D[2]);
    return (D[0] + D[4] + D[8]) + m2 + d3;
}

// GIMP domain update (domain.jl:1-52 via update.jl:7-28), after F <- ΔF F with the unscaled ΔF.
// ℓ from ℓ0 and the new F (det F, F_ii, U_ii of U = sqrt(F'F)) or from ℓ and ΔF (det ΔF, ΔF_ii,
// U_ii of sqrt(ΔF'ΔF)).  Both tensors come in as deviations from I, column-major DIM x DIM (D = ΔF -
// I, Fd = F - I), and every rule is applied as ℓ + ℓ (f - 1) with f - 1 formed without cancellation,
// so that the per-step rounding of the incremental rules stays far below the increment itself.
template <int DIM>
__device__ __forceinline__ void gimp_domain(const MCtx& A, int p, const float* D, const float* Fd) {
    const int how = A.cf.how;
    if (how == EP_HOW_UNDEFORMED || how == EP_HOW_NONE) return;
    const bool rel0 = how == EP_HOW_DETFIJ || how == EP_HOW_FII || how == EP_HOW_UII;   // from ℓ0
    const float* M = rel0 ? Fd : D;
    float fm1[3];
    if (how == EP_HOW_DETFIJ || how == EP_HOW_DETDFIJ) {
        const float j = DIM == 2 ? M[0] + M[3] + (M[0] * M[3] - M[2] * M[1]) : det1p_m1(M);
#pragma unroll
        for (int d = 0; d < DIM; ++d) fm1[d] = j;
    } else if (how == EP_HOW_FII || how == EP_HOW_DFII) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) fm1[d] = M[d + DIM * d];
    } else {
        // (I + M)'(I + M) - I = M + M' + M'M; U - I = Σ_k (sqrt(1 + μ_k) - 1) v_k v_k' over its
        // eigenpairs, sqrt(1 + μ) - 1 = μ / (1 + sqrt(1 + μ))
        float E[DIM][DIM];
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
            for (int j = 0; j < DIM; ++j) {
                float acc = M[j + DIM * i] + M[i + DIM * j];
#pragma unroll
                for (int k = 0; k < DIM; ++k) acc += M[k + DIM * i] * M[k + DIM * j];
                E[i][j] = acc;
            }
        if constexpr (DIM == 2) {
            const float m = 0.5f * (E[0][0] + E[1][1]), q = 0.5f * (E[0][0] - E[1][1]);
            const float r = sqrtf(q * q + E[0][1] * E[0][1]);
            const float mu1 = m + r, mu2 = m - r;
            const float s1 = mu1 / (1.f + sqrtf(1.f + mu1)), s2 = mu2 / (1.f + sqrtf(1.f + mu2));
            const float c2 = r > 0.f ? q / r : 1.f;   // cos 2θ of the first eigenvector
            fm1[0] = 0.5f * (s1 + s2) + 0.5f * (s1 - s2) * c2;
            fm1[1] = 0.5f * (s1 + s2) - 0.5f * (s1 - s2) * c2;
        } else {
            float a[3][3], v[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) a[i][j] = E[i][j];
            eig3f(a, v);
            float sk[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) sk[k] = a[k][k] / (1.f + sqrtf(1.f + a[k][k]));
#pragma unroll
            for (int d = 0; d < 3; ++d) fm1[d] = v[d][0] * v[d][0] * sk[0] + v[d][1] * v[d][1] * sk[1] + v[d][2] * v[d][2] * sk[2];
        }
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const float l = rel0 ? A.P.l0[d][p] : A.P.l[d][p];
        A.P.l[d][p] = l + l * fm1[d];
    }
}

// features of a finite-strain DP trial in the principal frame (ep_rmap.h layout, FP32):
// x[8], aux = (cos 2θ, sin 2θ, s, c); returns whether the trial leaves the DP surface
__device__ __forceinline__ bool rm_features32(float e11, float e22, float e12, float coh, float tphi, float Gc,
                                              float l2g, float* x, float* aux) {
    const float em = 0.5f * (e11 + e22), ed = 0.5f * (e11 - e22);
    const float r = sqrtf(ed * ed + e12 * e12);
    const float s = coh / (2.f * Gc);
    const float e1 = (em + r) / s, e2 = (em - r) / s;
    const float tr = e1 + e2;
    const float t1 = l2g * tr + e1, t2 = l2g * tr + e2;
    const float P = 0.5f * (t1 + t2), tII = 0.5f * (t1 - t2);
    const float den = sqrtf(9.f + 12.f * tphi * tphi);
    const float eta = 3.f * tphi / den, xi = 3.f / den;
    const float fs = tII + eta * P - xi;
    x[0] = e1; x[1] = e2; x[2] = 0.f; x[3] = coh * (float)(1.0 / RM_CREF);
    x[4] = tphi; x[5] = 0.f; x[6] = fmaxf(fs, 0.f); x[7] = 0.f;
    aux[0] = r > 0.f ? ed / r : 1.f;
    aux[1] = r > 0.f ? e12 / r : 0.f;
    aux[2] = s;
    aux[3] = coh;
    return (fs > 0.f && P < xi / eta) || P >= xi / eta;
}

// km_cons: F-bar scaling, F update, elastic predictor and return map, one lane per point.
// With the learned return map, a trial-yielding point is handed to the network (its
// features go to a slot; km_rmap_finish completes it); in record mode the exact map runs
// and the (features, exact label) pair of the point is appended to the record buffer.
// FLIP: the last block to finish flips the parity (km_flip's work, one launch less per step).
// cons_point: list slot k of the step (point p in cell c, stencil axes ax/az)
template <int BASIS, int ACC, bool ITER = false>
__device__ __forceinline__ void cons_point(const MCtx& A, int k, int p, int c, const Axis4& ax, const Axis4& az,
                                           int plastic_phase, int& nplastic, bool& emit, float* fx, float* fy,
                                           float* fa) {
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    {
        const float hx = (float)A.g.h[0], hz = (float)A.g.h[1];
        const float dtf = (float)A.ctl->dt;
        bool bad = false;
        const bool fin = A.cf.deform == EP_DEFORM_FINITE, lock = A.cf.locking;
        float wx[4], dwx[4], wz[4], dwz[4];
        // the half lengths of the step's shape functions (the domain update below rewrites ℓ)
        const float lx = BASIS == EP_BASIS_GIMPM ? A.P.l[0][p] : 0.f;
        const float lz = BASIS == EP_BASIS_GIMPM ? A.P.l[1][p] : 0.f;
        axis_w<BASIS>(ax, A.P.dx[cur][0][p], hx, 1.f / hx, lx, wx, dwx, bad);
        axis_w<BASIS>(az, A.P.dx[cur][1][p], hz, 1.f / hz, lz, wz, dwz, bad);
        float g00 = 0.f, g01 = 0.f, g10 = 0.f, g11 = 0.f, a = 0.f;
        if (lock) {
            // ∇v as the F-bar pass formed it for this slot; ΔJ̄ - 1 = Σ N δJ_n, δJ_n = z·w
            const float4 gs = A.P.gv[k];
            g00 = gs.x; g10 = gs.y; g01 = gs.z; g11 = gs.w;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (ax.cls[i] < 0) continue;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (az.cls[j] < 0) continue;
                    const float2 q = *reinterpret_cast<const float2*>(&A.N.vg4[node2(A.g, ax, az, i, j)].z);
                    a += wx[i] * wz[j] * (q.x * q.y);
                }
            }
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (ax.cls[i] < 0) continue;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (az.cls[j] < 0) continue;
                    const float Nx = dwx[i] * wz[j], Nz = wx[i] * dwz[j];
                    const float2 q = *reinterpret_cast<const float2*>(&A.N.vg4[node2(A.g, ax, az, i, j)]);
                    g00 += Nx * q.x;
                    g01 += Nz * q.x;
                    g10 += Nx * q.y;
                    g11 += Nz * q.y;
                }
            }
        }
        // D = ΔF - I = dt ∇v, column-major (deform.jl:13)
        float D[4] = {dtf * g00, dtf * g10, dtf * g01, dtf * g11};
        if (A.cf.trsfr == EP_TRSFR_TPIC) {
            A.P.dv[0][p] = g00; A.P.dv[1][p] = g10; A.P.dv[2][p] = g01; A.P.dv[3][p] = g11;
        }
        // F <- ΔF F with the unscaled ΔF (deform.jl:14): F += D F
        float Jm1 = 0.f;   // J - 1 (infinitesimal mass)
        float Fd[4];       // the new F - I (GIMP domain updates)
        if (ACC == 0) {
            const double F0 = A.P.Fd[0][p], F1 = A.P.Fd[1][p], F2 = A.P.Fd[2][p], F3 = A.P.Fd[3][p];
            const float f0 = (float)F0, f1 = (float)F1, f2 = (float)F2, f3 = (float)F3;
            const double N0 = F0 + (double)(D[0] * f0 + D[2] * f1);
            const double N1 = F1 + (double)(D[1] * f0 + D[3] * f1);
            const double N2 = F2 + (double)(D[0] * f2 + D[2] * f3);
            const double N3 = F3 + (double)(D[1] * f2 + D[3] * f3);
            A.P.Fd[0][p] = N0; A.P.Fd[1][p] = N1; A.P.Fd[2][p] = N2; A.P.Fd[3][p] = N3;
            Fd[0] = (float)(N0 - 1.0); Fd[1] = (float)N1; Fd[2] = (float)N2; Fd[3] = (float)(N3 - 1.0);
            if (!fin) Jm1 = (float)(N0 * N3 - N2 * N1 - 1.0);
        } else {
            float h0 = A.P.Fh[0][p], h1 = A.P.Fh[1][p], h2 = A.P.Fh[2][p], h3 = A.P.Fh[3][p];
            float l0 = A.P.Fl[0][p], l1 = A.P.Fl[1][p], l2 = A.P.Fl[2][p], l3 = A.P.Fl[3][p];
            const float i0 = D[0] * h0 + D[2] * h1, i1 = D[1] * h0 + D[3] * h1;
            const float i2 = D[0] * h2 + D[2] * h3, i3 = D[1] * h2 + D[3] * h3;
            df_add(h0, l0, i0); df_add(h1, l1, i1); df_add(h2, l2, i2); df_add(h3, l3, i3);
            A.P.Fh[0][p] = h0; A.P.Fh[1][p] = h1; A.P.Fh[2][p] = h2; A.P.Fh[3][p] = h3;
            A.P.Fl[0][p] = l0; A.P.Fl[1][p] = l1; A.P.Fl[2][p] = l2; A.P.Fl[3][p] = l3;
            // deviations from I formed exactly
            Fd[0] = (h0 - 1.f) + l0; Fd[1] = h1 + l1; Fd[2] = h2 + l2; Fd[3] = (h3 - 1.f) + l3;
            // J - 1 = (F11-1) + (F22-1) + (F11-1)(F22-1) - F12 F21
            if (!fin) Jm1 = Fd[0] + Fd[3] + (Fd[0] * Fd[3] - Fd[2] * Fd[1]);
        }
        if (!fin) {
            // infinitesimal: volume J Ω0 and mass ρ J Ω0 follow J (deform.jl:41-43)
            const float Om = A.P.Om0[p] + A.P.Om0[p] * Jm1;
            A.P.Om[p] = Om;
            A.P.mp[p] = A.P.rho[p] * Om;
        }
        if (BASIS == EP_BASIS_GIMPM) gimp_domain<2>(A, p, D, Fd);
        // F-bar: ΔF <- (ΔJ̄/ΔJ)^(1/2) ΔF, ΔJ̄ = Σ N ΔJ_n (volumetric.jl:23-36), increment form
        if (lock) {
            float sm1 = 0.f;      // Σ N - 1 over the existing nodes (GIMP next to a mesh edge)
            if (BASIS == EP_BASIS_GIMPM) {
                const float mx = axis_miss<BASIS>(ax, A.P.dx[cur][0][p], hx, lx);
                const float mz = axis_miss<BASIS>(az, A.P.dx[cur][1][p], hz, lz);
                sm1 = -(mx + mz) + mx * mz;
            }
            const float dJp = D[0] + D[3] + (D[0] * D[3] - D[2] * D[1]);
            const float r1 = (sm1 + a - dJp) / (1.f + dJp);    // ΔJ̄/ΔJ - 1
            const float s1 = r1 / (1.f + sqrtf(1.f + r1));     // sqrt(1 + r1) - 1
            D[0] = D[0] * (1.f + s1) + s1;
            D[1] = D[1] * (1.f + s1);
            D[2] = D[2] * (1.f + s1);
            D[3] = D[3] * (1.f + s1) + s1;
        }
        float tt[3];
        float te11 = 0.f, te22 = 0.f, te12 = 0.f;   // trial log strain (finite)
        if (fin) {
            // b <- ΔF b ΔF' = b + (D b + b D' + D b D') (elast.jl:49), then ε = ½ log b (elast.jl:51-52)
            float b11, b22, b12, mu, dd, qq;
            if (ACC == 0) {
                double B0 = A.P.bd[0][p], B1 = A.P.bd[1][p], B2 = A.P.bd[2][p];
                b11 = (float)B0; b22 = (float)B1; b12 = (float)B2;
                const float M00 = D[0] * b11 + D[2] * b12, M01 = D[0] * b12 + D[2] * b22;
                const float M10 = D[1] * b11 + D[3] * b12, M11 = D[1] * b12 + D[3] * b22;
                B0 += (double)(2.f * M00 + (M00 * D[0] + M01 * D[2]));
                B1 += (double)(2.f * M11 + (M10 * D[1] + M11 * D[3]));
                B2 += (double)(M10 + M01 + (M00 * D[1] + M01 * D[3]));
                A.P.bd[0][p] = B0; A.P.bd[1][p] = B1; A.P.bd[2][p] = B2;
                const double m = 0.5 * (B0 + B1);
                dd = (float)(0.5 * (B0 - B1));
                qq = (float)B2;
                mu = (float)(m - 1.0);
                // log m in FP64 (the isotropic part of log b_e)
                tt[0] = (float)ep_log(m);
            } else {
                float h0 = A.P.bh[0][p], h1 = A.P.bh[1][p], h2 = A.P.bh[2][p];
                float l0 = A.P.bl[0][p], l1 = A.P.bl[1][p], l2 = A.P.bl[2][p];
                b11 = h0; b22 = h1; b12 = h2;
                const float M00 = D[0] * b11 + D[2] * b12, M01 = D[0] * b12 + D[2] * b22;
                const float M10 = D[1] * b11 + D[3] * b12, M11 = D[1] * b12 + D[3] * b22;
                df_add(h0, l0, 2.f * M00 + (M00 * D[0] + M01 * D[2]));
                df_add(h1, l1, 2.f * M11 + (M10 * D[1] + M11 * D[3]));
                df_add(h2, l2, M10 + M01 + (M00 * D[1] + M01 * D[3]));
                A.P.bh[0][p] = h0; A.P.bh[1][p] = h1; A.P.bh[2][p] = h2;
                A.P.bl[0][p] = l0; A.P.bl[1][p] = l1; A.P.bl[2][p] = l2;
                // deviations from 1 formed exactly from the pairs (h - 1 is exact near 1)
                mu = 0.5f * (((h0 - 1.f) + (h1 - 1.f)) + (l0 + l1));
                dd = 0.5f * ((h0 - h1) + (l0 - l1));
                qq = h2 + l2;
                tt[0] = log1pf(mu);   // log m, m = 1 + μ
            }
            const float mf = 1.f + mu;
            const float x2 = (dd * dd + qq * qq) / (mf * mf);
            const float L0 = tt[0] + 0.5f * log1pf(-x2);
            const float kd = atanh_over_x(x2) / mf;
            te11 = 0.5f * (L0 + kd * dd);
            te22 = 0.5f * (L0 - kd * dd);
            te12 = 0.5f * kd * qq;
            const float v2 = 2.f * te12;
            tt[0] = A.Del[0] * te11 + A.Del[3] * te22 + A.Del[6] * v2;
            tt[1] = A.Del[1] * te11 + A.Del[4] * te22 + A.Del[7] * v2;
            tt[2] = A.Del[2] * te11 + A.Del[5] * te22 + A.Del[8] * v2;
        } else {
            // σ += Del voigt(sym(ΔF) - I, 2) (+ ωσ - σω for the objective rate) (elast.jl:73-78)
            tt[0] = A.P.tau[0][p]; tt[1] = A.P.tau[1][p]; tt[2] = A.P.tau[2][p];
            const float e11 = D[0], e22 = D[3], g12 = D[1] + D[2];
            float d0 = A.Del[0] * e11 + A.Del[3] * e22 + A.Del[6] * g12;
            float d1 = A.Del[1] * e11 + A.Del[4] * e22 + A.Del[7] * g12;
            float d2 = A.Del[2] * e11 + A.Del[5] * e22 + A.Del[8] * g12;
            if (A.cf.jaumann) {
                const float w = 0.5f * (D[2] - D[1]);
                d0 += 2.f * w * tt[2];
                d1 -= 2.f * w * tt[2];
                d2 += w * (tt[1] - tt[0]);
            }
            tt[0] += d0; tt[1] += d1; tt[2] += d2;
        }
        if (plastic_phase) {
            float ep1f = ACC == 0 ? (float)A.P.ep1d[p] : A.P.ep1h[p] + A.P.ep1l[p];
            const float ep2 = A.cf.nonloc ? A.P.ep2[p] : ep1f;
            bool yielded = false, deferred = false;
            float inc = 0.f, newg = 0.f;
            bool absolute = false;
            if (A.cf.cons == EP_CONS_DP) {
                if (A.rmode != EP_RMAP_EXACT && fin) {
                    const float coh = fmaxf(A.P.c0[p] + A.Hp * ep2, A.P.cr[p]);
                    const bool ytr = rm_features32(te11, te22, te12, coh, A.P.tphi[p], A.Gc, A.l2g, fx, fa);
                    deferred = ytr && A.rmode == EP_RMAP_LEARNED;
                }
                if (deferred) {
                    emit = true;              // km_rmap_finish writes τ, Δλ, ϵpII and b_e
                    ++nplastic;
                } else {
                    const float dl = dp32(tt, ep2, A.P.c0[p], A.P.cr[p], A.P.tphi[p], A.Hp, A.Kc, A.Gc, &inc);
                    A.P.dlam[p] = dl;
                    yielded = dl != 0.f;
                    if (yielded && A.rmode == EP_RMAP_RECORD && fin) emit = rm_label(fx, (double)A.l2g, fy) != 0;
                }
            } else if constexpr (!ITER) {
                const float Dl[9] = {A.Del[0], A.Del[1], A.Del[2], A.Del[3], A.Del[4],
                                     A.Del[5], A.Del[6], A.Del[7], A.Del[8]};
                yielded = j232(tt, ep2, A.P.c0[p], A.P.cr[p], A.Hp, Dl, &newg) != 0;
                absolute = true;
            } else {
                // MC / modified Cam-Clay (the ITER instantiations only, so that the DP and J2 kernels
                // carry no call): the iterative returns run as FP64 islands (ep_scalar.h) on the FP32
                // trial stress; their absolute tolerances (1e-6 Pa, Pa²) are below FP32 resolution
                newg = cons_iterative<3>(A, p, tt, ep2, &yielded);
                absolute = true;
            }
            if (yielded) {
                ++nplastic;
                if (absolute) {
                    if (ACC == 0) {
                        A.P.ep1d[p] = (double)newg;
                    } else {
                        A.P.ep1h[p] = newg;
                        A.P.ep1l[p] = 0.f;
                    }
                } else {
                    add_ep1<ACC>(A, p, inc);
                }
                if (fin) {
                    // ε = tensor(Del \ τ, ½); b = exp(2ε) (DP.jl:63-66)
                    const float e11 = A.Cmp[0] * tt[0] + A.Cmp[3] * tt[1] + A.Cmp[6] * tt[2];
                    const float e22 = A.Cmp[1] * tt[0] + A.Cmp[4] * tt[1] + A.Cmp[7] * tt[2];
                    const float e12 = 0.5f * (A.Cmp[2] * tt[0] + A.Cmp[5] * tt[1] + A.Cmp[8] * tt[2]);
                    rebuild_b<ACC>(A, p, e11, e22, e12);
                }
            }
        }
        A.P.tau[0][p] = tt[0];
        A.P.tau[1][p] = tt[1];
        A.P.tau[2][p] = tt[2];
        if (!(isfinite(tt[0]) && isfinite(tt[1]) && isfinite(tt[2]))) set_err(A.ctl, EP_ERR_NONFINITE, p);
        if (!lock) place_next(A, p, nxt);
        if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, c);
    }
}

// the warp's emitted slots of km_cons: learned-map slots or recorded pairs, one atomic per warp
__device__ __forceinline__ void cons_emit(const MCtx& A, bool emit, const float* fx, const float* fy, const float* fa,
                                          int fp) {
    // learned map slots / recorded pairs: one atomic per warp for the warp's points
    if (A.rmode != EP_RMAP_EXACT) {
        const unsigned bal = __ballot_sync(0xffffffffu, emit);
        if (bal) {
            const int lane = threadIdx.x & 31;
            const unsigned below = bal & ((1u << lane) - 1u);
            if (A.rmode == EP_RMAP_LEARNED) {
                int base = 0;
                if (lane == 0) base = atomicAdd(A.rcount, __popc(bal));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (emit) {
                    const int slot = base + __popc(below);
                    float4* dx = reinterpret_cast<float4*>(A.rx + (size_t)slot * RM_NX);
                    dx[0] = make_float4(fx[0], fx[1], fx[2], fx[3]);
                    dx[1] = make_float4(fx[4], fx[5], fx[6], fx[7]);
                    *reinterpret_cast<float4*>(A.raux + (size_t)slot * 4) = make_float4(fa[0], fa[1], fa[2], fa[3]);
                    A.rpt[slot] = fp;
                }
            } else {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd((unsigned long long*)A.rec_count, (unsigned long long)__popc(bal));
                base = __shfl_sync(0xffffffffu, base, 0);
                const long long slot = (long long)base + __popc(below);
                if (emit && slot < A.rec_cap) {
                    float4* dx = reinterpret_cast<float4*>(A.rx + (size_t)slot * RM_NX);
                    dx[0] = make_float4(fx[0], fx[1], fx[2], fx[3]);
                    dx[1] = make_float4(fx[4], fx[5], fx[6], fx[7]);
                    *reinterpret_cast<float4*>(A.ry + (size_t)slot * RM_NY) = make_float4(fy[0], fy[1], fy[2], fy[3]);
                }
            }
        }
    }
}

// the plastic count (one atomic per warp) and, with FLIP, the parity flip by the last block to finish
template <bool FLIP>
__device__ __forceinline__ void cons_finish(const MCtx& A, int nplastic) {
    const int tot = __reduce_add_sync(0xffffffffu, nplastic);
    if ((threadIdx.x & 31) == 0 && tot) atomicAdd((unsigned long long*)&A.ctl->plastic, (unsigned long long)tot);
    if (FLIP) {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(&A.S.sync[1], 1) == (int)gridDim.x - 1) A.ctl->parity ^= 1;
        }
    }
}

// km_cons over the sorted list, one lane per slot
template <int BASIS, int ACC, bool FLIP = false, bool ITER = false>
__device__ __forceinline__ void cons_body(const MCtx& A, int bid, int plastic_phase) {
    EP_ACTIVE(A.ctl);
    const int cur = A.ctl->parity;
    const int k = bid * blockDim.x + threadIdx.x;
    int nplastic = 0;
    bool emit = false;
    float fx[RM_NX], fy[RM_NY], fa[4];
    int fp = 0;
    if (k < A.S.start[cur][A.g.ncell]) {
        const int p = A.S.list[cur][k], c = A.S.cellof[cur][k];
        fp = p;
        const int ex = c / A.g.nel[1], ez = c - ex * A.g.nel[1];
        const Axis4 ax = axis4(A.g, 0, ex), az = axis4(A.g, 1, ez);
        cons_point<BASIS, ACC, ITER>(A, k, p, c, ax, az, plastic_phase, nplastic, emit, fx, fy, fa);
    }
    cons_emit(A, emit, fx, fy, fa, fp);
    cons_finish<FLIP>(A, nplastic);
}

template <int BASIS, int ACC, bool FLIP = false, bool ITER = false>
__global__ void __launch_bounds__(256, 4) km_cons(MCtx A, int plastic_phase) {
    pdl_enter();
    cons_body<BASIS, ACC, FLIP, ITER>(A, blockIdx.x, plastic_phase);
}


// rmap_fallback_slot32: the rejected slots' return as the exact-map mixed step runs it (dp32: the
// Drucker-Prager return of DP.jl:33-66 in FP32, on the trial rebuilt from the slot; b_e = exp(2 Del \ τ)
// by rebuild_b): the same result a point gets without the network.  A few slots in most CTAs of the
// finish kernel are rejected, so the FP64 form's one-lane chain set the kernel's duration.
template <int ACC>
__device__ __noinline__ void rmap_fallback_slot32(const MCtx& A, int i) {
    const float4 x0 = *reinterpret_cast<const float4*>(A.rx + (size_t)i * RM_NX);
    const float4 x1 = *reinterpret_cast<const float4*>(A.rx + (size_t)i * RM_NX + 4);
    const float4 ax = *reinterpret_cast<const float4*>(A.raux + (size_t)i * 4);
    const int p = A.rpt[i];
    const float c2 = ax.x, s2 = ax.y, s = ax.z, coh = ax.w;
    const float q1 = s * x0.x, q2 = s * x0.y;
    const float em = 0.5f * (q1 + q2), r = 0.5f * (q1 - q2);
    const float te[3] = {em + r * c2, em - r * c2, 2.f * r * s2};
    float tt[3];
    for (int a = 0; a < 3; ++a) tt[a] = A.Del[a] * te[0] + A.Del[a + 3] * te[1] + A.Del[a + 6] * te[2];
    float inc = 0.f;
    const float dl = dp32(tt, 0.f, coh, 0.f, x1.x, 0.f, A.Kc, A.Gc, &inc);
    A.P.dlam[p] = dl;
    add_ep1<ACC>(A, p, inc);
    if (dl != 0.f) {
        const float e11 = A.Cmp[0] * tt[0] + A.Cmp[3] * tt[1] + A.Cmp[6] * tt[2];
        const float e22 = A.Cmp[1] * tt[0] + A.Cmp[4] * tt[1] + A.Cmp[7] * tt[2];
        const float e12 = 0.5f * (A.Cmp[2] * tt[0] + A.Cmp[5] * tt[1] + A.Cmp[8] * tt[2]);
        rebuild_b<ACC>(A, p, e11, e22, e12);
    }
    A.P.tau[0][p] = tt[0];
    A.P.tau[1][p] = tt[1];
    A.P.tau[2][p] = tt[2];
    if (!(isfinite(tt[0]) && isfinite(tt[1]) && isfinite(tt[2]))) set_err(A.ctl, EP_ERR_NONFINITE, p);
}

// km_rmap_finish: the network's returned strains for the slots of km_cons, accepted when
// the trial lies on the compressive side of the apex, the returned stress is on the yield
// surface and keeps the trial mean stress (both within 1e-3 c), the principal order is
// kept and Δλ >= 0; the other slots go to the exact return (DP.jl:33-66, rmap_fallback_slot32)
// FLIP: the last block to finish does km_flip's work (parity flip, slot counters emptied)
template <int ACC, bool FLIP = false>
__global__ void __launch_bounds__(256) km_rmap_finish(MCtx A) {
    EP_ACTIVE(A.ctl);
    const int n = *A.rcount;
    int nl = 0, nf = 0;
    // grid-stride over the slots (the count is on the device; the grid is a few CTAs per SM)
    for (int i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
    const int i = i0 + threadIdx.x;
    bool reject = false;
    if (i < n) {
        const float4 x0 = *reinterpret_cast<const float4*>(A.rx + (size_t)i * RM_NX);
        const float4 x1 = *reinterpret_cast<const float4*>(A.rx + (size_t)i * RM_NX + 4);
        const float4 y = *reinterpret_cast<const float4*>(A.ry + (size_t)i * RM_NY);
        const float4 ax = *reinterpret_cast<const float4*>(A.raux + (size_t)i * 4);
        const float c2 = ax.x, s2 = ax.y, s = ax.z, coh = ax.w;
        const float tphi = x1.x, phin = x1.z;
        const float den = sqrtf(9.f + 12.f * tphi * tphi), eta = 3.f * tphi / den, xi = 3.f * coh / den;
        bool ok = phin >= (float)RM_PHI_MIN && isfinite(y.x) && isfinite(y.y);
        float tt[3] = {0.f, 0.f, 0.f}, e11 = 0.f, e22 = 0.f, e12 = 0.f, dl = 0.f;
        if (ok) {
            float y0 = y.x, y1 = y.y;
            if (x1.y == 0.f) {
                // tan ψ = 0: the exact return's plastic strain increment is deviatoric, so the
                // volumetric part of the predicted correction is removed (it would accumulate in
                // the mean stress, which no later return corrects)
                const float yd = 0.5f * (y0 - y1);
                y0 = yd;
                y1 = -yd;
            }
            const float e1 = s * (x0.x + phin * y0), e2 = s * (x0.y + phin * y1);
            const float em = 0.5f * (e1 + e2), r = 0.5f * (e1 - e2);
            e11 = em + r * c2;
            e22 = em - r * c2;
            e12 = r * s2;
            const float v2 = 2.f * e12;
            tt[0] = A.Del[0] * e11 + A.Del[3] * e22 + A.Del[6] * v2;
            tt[1] = A.Del[1] * e11 + A.Del[4] * e22 + A.Del[7] * v2;
            tt[2] = A.Del[2] * e11 + A.Del[5] * e22 + A.Del[8] * v2;
            const float P = 0.5f * (tt[0] + tt[1]), d0 = tt[0] - P, d1 = tt[1] - P;
            const float tII = sqrtf(0.5f * (d0 * d0 + d1 * d1) + tt[2] * tt[2]);
            const float fs = tII + eta * P - xi;
            dl = (0.5f * coh * (x0.x - x0.y) - tII) / A.Gc;    // Δλ = (τII,trial - τII) / G (ψ = 0)
            // ψ = 0 makes the plastic strain increment deviatoric (DP.jl:37, 47-52): the returned
            // mean stress is the trial one, P_trial = c (λ/2G + 1/2)(x0 + x1)
            const float Ptr = coh * (A.l2g + 0.5f) * (x0.x + x0.y);
            // beyond the apex (P >= σm = c / tan ϕ) the exact map may take its tension-apex branch,
            // which moves the mean stress (DP.jl:53-58): those trials always go to the exact map
            const bool below_apex = tphi > 0.f ? Ptr < coh / tphi : true;
            ok = fabsf(fs) <= 1.0e-3f * coh && fabsf(P - Ptr) <= 1.0e-3f * coh && dl >= 0.f && r >= 0.f &&
                 below_apex && isfinite(fs);
        }
        if (ok) {
            ++nl;
            const int p = A.rpt[i];
            add_ep1<ACC>(A, p, dl * 0.57735026918962576f);
            A.P.dlam[p] = dl;
            rebuild_b<ACC>(A, p, e11, e22, e12);
            A.P.tau[0][p] = tt[0];
            A.P.tau[1][p] = tt[1];
            A.P.tau[2][p] = tt[2];
        } else {
            reject = true;
        }
    }
    // rejected slots: the exact return right here (a few per thousand slots, in FP32 as the exact-map
    // step runs it)
    if (reject) {
        rmap_fallback_slot32<ACC>(A, i);
        ++nf;
    }
    }
    const int tl = __reduce_add_sync(0xffffffffu, nl), tf = __reduce_add_sync(0xffffffffu, nf);
    if ((threadIdx.x & 31) == 0 && tl) atomicAdd(&A.ctl->rm_learned, (unsigned long long)tl);
    if ((threadIdx.x & 31) == 0 && tf) atomicAdd(&A.ctl->rm_fallback, (unsigned long long)tf);
    if (FLIP) {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(&A.S.sync[2], 1) == (int)gridDim.x - 1) {
                A.ctl->parity ^= 1;
                *A.rcount = 0;
                if (A.fbcount) *A.fbcount = 0;
            }
        }
    }
}

__global__ void km_flip(Ctl* ctl, int* rcount, int* fbcount) {
    if (!ctl->active) return;
    ctl->parity ^= 1;
    if (rcount) *rcount = 0;   // learned map slots and fallbacks of the next step
    if (fbcount) *fbcount = 0;
}


// ---------------------------------------------------------------------------
// km_nonlocal: nonlocal averaging of ϵpII in the reference's serial visiting order
// (nonlocal.jl:18-47 with plast.jl:51-59), one warp per point, 2d.  Same sums as the FP64
// step (for a point p with Δλ != 0 from the previous return and N(p) the points of the
// cells within ±ceil(ls/h) of p's cell at the step start):
//   W[p]  = Σ_{r in N(p), r plastic, r < p} ω(r,p) + Σ_{q in N(p), not (q plastic and q < p)} ω(p,q)
//   ϵ2[p] = Σ_{q in N(p), not (q plastic and q < p)} (ω(p,q) / W[p]) ϵ1[q]
// in ascending id order, ω = (d/ls) exp(-(d/ls)^2), d from the positions after G2P (cell
// node coordinate in FP64 + FP32 offset); ϵ2 = ϵ1 when W <= 1e-16, 0 for non-plastic points.
constexpr int NLM_CAP = 2048;

template <int ACC>
__device__ __forceinline__ float ep1_of(const MCtx& A, int q) {
    return ACC == 0 ? (float)A.P.ep1d[q] : A.P.ep1h[q] + A.P.ep1l[q];
}

template <int ACC>
__global__ void __launch_bounds__(32) km_nonlocal(MCtx A) {
    EP_ACTIVE(A.ctl);
    __shared__ int qs[NLM_CAP];
    __shared__ float om[NLM_CAP];
    const int p = blockIdx.x, lane = threadIdx.x;
    if (p >= A.P.np) return;
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int cp = A.P.pcell[cur][p], cn = A.P.pcell[nxt][p];
    if (A.P.dlam[p] == 0.f || cp < 0 || cn < 0) {
        if (lane == 0) A.P.ep2[p] = 0.f;
        return;
    }
    const int n1 = A.g.nel[1];
    const int ex = cp / n1, ez = cp - ex * n1;
    const int lo0 = max(ex - A.g.nnel[0], 0), hi0 = min(ex + A.g.nnel[0], A.g.nel[0] - 1);
    const int lo1 = max(ez - A.g.nnel[1], 0), hi1 = min(ez + A.g.nnel[1], n1 - 1);
    const int* start = A.S.start[cur];
    const int* list = A.S.list[cur];
    int L = 0;
    for (int a = lo0; a <= hi0; ++a) L += start[hi1 + n1 * a + 1] - start[lo1 + n1 * a];
    const double ls = A.cf.ls;
    const int exn = cn / n1, ezn = cn - exn * n1;
    const double xp0 = A.g.ax[0][exn] + (double)A.P.dx[nxt][0][p];
    const double xp1 = A.g.ax[1][ezn] + (double)A.P.dx[nxt][1][p];
    auto omega = [&](int q) {
        const int cq = A.P.pcell[nxt][q];
        const int eq = cq / n1, fq = cq - eq * n1;
        const double xi = xp0 - (A.g.ax[0][eq] + (double)A.P.dx[nxt][0][q]);
        const double et = xp1 - (A.g.ax[1][fq] + (double)A.P.dx[nxt][1][q]);
        const float r = (float)(sqrt(xi * xi + et * et) / ls);
        return r * expf(-(r * r));
    };
    if (L <= NLM_CAP) {
        // candidate ids in cell order (each column's cells are one contiguous slice of the list)
        int pos = 0;
        for (int a = lo0; a <= hi0; ++a) {
            const int b = start[lo1 + n1 * a], n = start[hi1 + n1 * a + 1] - b;
            for (int k = lane; k < n; k += 32) qs[pos + k] = list[b + k];
            pos += n;
        }
        int P2 = 32;
        while (P2 < L) P2 <<= 1;
        for (int k = L + lane; k < P2; k += 32) qs[k] = INT_MAX;
        __syncwarp();
        // bitonic sort into ascending point id (the reference's serial order)
        for (int k = 2; k <= P2; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int t = lane; t < P2; t += 32) {
                    const int q = t ^ j;
                    if (q > t) {
                        const int a = qs[t], c = qs[q];
                        const bool asc = (t & k) == 0;
                        if ((a > c) == asc) {
                            qs[t] = c;
                            qs[q] = a;
                        }
                    }
                }
                __syncwarp();
            }
        for (int t = lane; t < L; t += 32) om[t] = omega(qs[t]);
        __syncwarp();
        if (lane == 0) {
            float W = 0.f;
            for (int t = 0; t < L; ++t) {
                const int q = qs[t];
                if (q >= p) break;
                if (A.P.dlam[q] != 0.f) W += om[t];
            }
            for (int t = 0; t < L; ++t) {
                const int q = qs[t];
                if (q < p && A.P.dlam[q] != 0.f) continue;
                W += om[t];
            }
            float s = 0.f;
            if (!(W > 1e-16f)) {
                s = ep1_of<ACC>(A, p);
            } else {
                for (int t = 0; t < L; ++t) {
                    const int q = qs[t];
                    if (q < p && A.P.dlam[q] != 0.f) continue;
                    s += (om[t] / W) * ep1_of<ACC>(A, q);
                }
            }
            A.P.ep2[p] = s;
        }
        return;
    }
    // more candidates than the shared buffer holds: walk them in ascending order by repeated
    // minimum selection (slow, same sums)
    if (lane != 0) return;
    float W = 0.f;
    for (int pass = 0; pass < 3; ++pass) {
        float s = 0.f;
        int last = -1;
        if (pass == 2 && !(W > 1e-16f)) {
            A.P.ep2[p] = ep1_of<ACC>(A, p);
            return;
        }
        while (true) {
            int best = INT_MAX;
            for (int a = lo0; a <= hi0; ++a)
                for (int k = start[lo1 + n1 * a]; k < start[hi1 + n1 * a + 1]; ++k) {
                    const int q = list[k];
                    if (q > last && q < best) best = q;
                }
            if (best == INT_MAX) break;
            last = best;
            const int q = best;
            const bool plq = A.P.dlam[q] != 0.f;
            if (pass == 0 && !(q < p && plq)) continue;
            if (pass >= 1 && (q < p && plq)) continue;
            const float w = omega(q);
            if (pass < 2) W += w;
            else s += (w / W) * ep1_of<ACC>(A, q);
        }
        if (pass == 2) A.P.ep2[p] = s;
    }
}

// ---------------------------------------------------------------------------
// exclusive scan of count[nxt] into start[nxt] (parity read on the device)
constexpr int MSCAN_BS = 1024, MSCAN_IPT = 4, MSCAN_CHUNK = MSCAN_BS * MSCAN_IPT;

__device__ __forceinline__ int mwarp_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

__device__ __forceinline__ int mblock_scan(int v, int* tot) {
    __shared__ int ws[33];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int inc = mwarp_scan(v);
    if (lane == 31) ws[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int s = lane < nw ? ws[lane] : 0;
        int si = mwarp_scan(s);
        if (lane < nw) ws[lane] = si - s;
        if (lane == 31) ws[32] = si;
    }
    __syncthreads();
    int r = ws[wid] + inc - v;
    *tot = ws[32];
    __syncthreads();
    return r;
}

// which = 0: scan count[nxt] -> start[nxt] (inside a step); 1: count[cur] -> start[cur] (set-up)
__global__ void km_scan_local(MCtx A, int which, int* bsum) {
    if (which == 0 && !A.ctl->active) return;
    const int par = which == 0 ? (A.ctl->parity ^ 1) : A.ctl->parity;
    const int n = A.g.ncell;
    const int* in = A.S.count[par];
    int* out = A.S.start[par];
    const int base = blockIdx.x * MSCAN_CHUNK + threadIdx.x * MSCAN_IPT;
    int v[MSCAN_IPT], s = 0;
#pragma unroll
    for (int i = 0; i < MSCAN_IPT; ++i) {
        v[i] = base + i < n ? in[base + i] : 0;
        s += v[i];
    }
    int tot;
    int ex = mblock_scan(s, &tot);
#pragma unroll
    for (int i = 0; i < MSCAN_IPT; ++i) {
        if (base + i < n) out[base + i] = ex;
        ex += v[i];
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void km_scan_sums(MCtx A, int which, int* bsum, int nb) {
    if (which == 0 && !A.ctl->active) return;
    const int par = which == 0 ? (A.ctl->parity ^ 1) : A.ctl->parity;
    const int base = threadIdx.x * MSCAN_IPT;
    int v[MSCAN_IPT], s = 0;
#pragma unroll
    for (int i = 0; i < MSCAN_IPT; ++i) {
        v[i] = base + i < nb ? bsum[base + i] : 0;
        s += v[i];
    }
    int tot;
    int ex = mblock_scan(s, &tot);
#pragma unroll
    for (int i = 0; i < MSCAN_IPT; ++i) {
        if (base + i < nb) bsum[base + i] = ex;
        ex += v[i];
    }
    if (threadIdx.x == 0) A.S.start[par][A.g.ncell] = tot;
}

__global__ void km_scan_add(MCtx A, int which, const int* bsum) {
    if (which == 0 && !A.ctl->active) return;
    const int par = which == 0 ? (A.ctl->parity ^ 1) : A.ctl->parity;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A.g.ncell) A.S.start[par][i] += bsum[i / MSCAN_CHUNK];
}

// ---------------------------------------------------------------------------
// km_zero: the step-start zeroing of the node accumulators (m, p, f) and of the counts, cursor and
// scan words, as a kernel so that steps past the end of a window (EP_ACTIVE) leave the last step's
// nodal fields in place for download.
// begin_step = 1: the kernel also starts the step the way k_ctl_begin_step does (active unless an error
// was raised, vmax and the plastic count reset), so that a one-step graph needs no launch for it; the
// kernels after it read the control block only once it has finished.  Both regions start 16-byte
// aligned (their own allocations): 16-byte stores, then the tails.
__global__ void __launch_bounds__(256) km_zero(MCtx A, float* g, long long ng, int* z, long long nz, int begin_step) {
    pdl_enter();
    if (begin_step) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            Ctl* c = A.ctl;
            c->active = c->err ? 0 : 1;
            for (int i = 0; i < 3; ++i) c->vmax_bits[i] = 0ull;
            c->plastic = 0;
        }
    } else {
        EP_ACTIVE(A.ctl);
    }
    const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, st = (long long)gridDim.x * blockDim.x;
    const float4 f0 = make_float4(0.f, 0.f, 0.f, 0.f);
    const int4 z0 = make_int4(0, 0, 0, 0);
    for (long long i = i0; i < ng / 4; i += st) reinterpret_cast<float4*>(g)[i] = f0;
    for (long long i = i0; i < nz / 4; i += st) reinterpret_cast<int4*>(z)[i] = z0;
    if (i0 < (ng & 3)) g[(ng & ~3LL) + i0] = 0.f;
    if (i0 < (nz & 3)) z[(nz & ~3LL) + i0] = 0;
}

// km_vmusl_scan: in one launch, the mUSL nodal velocity (vmusl_body, blocks past the scan tiles) and
// the exclusive scan count[nxt] -> start[nxt] (the next step's cell offsets, total at ncell) as a
// single-pass scan with decoupled look-back: a block takes the next tile by ticket, publishes its
// aggregate, adds its predecessors' published aggregates (32 per round, one warp) until it meets an
// inclusive prefix, and publishes its own.  Tickets hand tiles out in launch order, so a block only waits for tiles that
// started before it; every wait is bounded and reports EP_ERR_TIMEOUT if it gives up.
constexpr unsigned long long SCAN_AGG = 1ull << 32, SCAN_PREFIX = 2ull << 32;
constexpr int MSCAN2_BS = 512, MSCAN2_IPT = MSCAN_TILE / MSCAN2_BS;

__device__ __forceinline__ unsigned long long ld_status(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__global__ void __launch_bounds__(MSCAN2_BS) km_vmusl_scan(MCtx A, int ntiles) {
    pdl_enter();
    EP_ACTIVE(A.ctl);
    if ((int)blockIdx.x >= ntiles) {
        // the mUSL velocity over MSCAN2_BS nodes per block
        const int n = (blockIdx.x - ntiles) * MSCAN2_BS + threadIdx.x;
        if (n < A.g.nnode) vmusl_one(A, n);
        return;
    }
    __shared__ int tile_s, excl_s;
    const int par = A.ctl->parity ^ 1;
    const int nc = A.g.ncell;
    if (threadIdx.x == 0) tile_s = atomicAdd(&A.S.sync[0], 1);
    __syncthreads();
    const int tile = tile_s;
    const int* in = A.S.count[par];
    int* out = A.S.start[par];
    const int base = tile * MSCAN_TILE + threadIdx.x * MSCAN2_IPT;
    int v[MSCAN2_IPT], sum = 0;
#pragma unroll
    for (int i = 0; i < MSCAN2_IPT; ++i) {
        v[i] = base + i < nc ? in[base + i] : 0;
        sum += v[i];
    }
    int agg;
    const int ex = mblock_scan(sum, &agg);
    if (threadIdx.x < 32) {
        // look-back by the first warp, 32 predecessors per round: lane i reads tile - 1 - i - 32 r; the
        // nearest published prefix ends the walk, and the aggregates up to it are summed
        const int lane = threadIdx.x;
        unsigned long long* st = A.S.scan_status;
        int excl = 0;
        if (lane == 0) atomicExch(&st[tile], (tile == 0 ? SCAN_PREFIX : SCAN_AGG) | (unsigned)agg);
        int j0 = tile - 1;
        long long spins = 0;
        while (j0 >= 0) {
            const int j = j0 - lane;
            const unsigned long long w = j >= 0 ? ld_status(&st[j]) : SCAN_PREFIX;   // before tile 0: prefix 0
            const unsigned long long flag = w & 0xffffffff00000000ull;
            const unsigned pre = __ballot_sync(0xffffffffu, flag == SCAN_PREFIX);
            const unsigned none = __ballot_sync(0xffffffffu, flag == 0);
            const int first = pre ? __ffs(pre) - 1 : 32;                 // nearest predecessor with a prefix
            const unsigned need = first < 31 ? (2u << first) - 1u : 0xffffffffu;
            if (none & need) {
                if (++spins > (1ll << 22)) {          // ~1 s of waiting: give up and report it
                    if (lane == 0) set_err(A.ctl, EP_ERR_TIMEOUT, tile);
                    break;
                }
                __nanosleep(32);
                continue;
            }
            int v = lane <= first ? (int)(unsigned)(w & 0xffffffffull) : 0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            excl += v;
            if (first < 32) break;
            j0 -= 32;
        }
        if (lane == 0) {
            if (tile > 0) atomicExch(&st[tile], SCAN_PREFIX | (unsigned)(excl + agg));
            excl_s = excl;
            if (tile == ntiles - 1) out[nc] = excl + agg;
        }
    }
    __syncthreads();
    int e = excl_s + ex;
#pragma unroll
    for (int i = 0; i < MSCAN2_IPT; ++i) {
        if (base + i < nc) out[base + i] = e;
        e += v[i];
    }
}

static int mixed_scan(const MCtx& A, int which, int* bsum, cudaStream_t s) {
    const int n = A.g.ncell, nb = (n + MSCAN_CHUNK - 1) / MSCAN_CHUNK;
    km_scan_local<<<nb, MSCAN_BS, 0, s>>>(A, which, bsum);
    km_scan_sums<<<1, MSCAN_BS, 0, s>>>(A, which, bsum, nb);
    if (nb > 1) km_scan_add<<<(n + 255) / 256, 256, 0, s>>>(A, which, bsum);
    return nb > 1 ? 3 : 2;
}

// SMs of the current device (grids of the slot kernels, whose counts live on the device)
static int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
            n = v;
        if (n <= 0) n = 1;
    }
    return n;
}

// the largest node box of the tiles of TC cells (tile_box), for the choice of the fused grid update
static int max_tile_box(const Geo& g, int TC) {
    int mx = 0;
    for (int c0 = 0; c0 < g.ncell; c0 += TC) {
        int NX;
        const TileBox b = tile_box(g, c0, std::min(c0 + TC, g.ncell), NX, INT_MAX);
        mx = std::max(mx, NX * b.NZ);
    }
    return mx;
}

// Launch with programmatic stream serialization (the kernel calls pdl_enter() first), so that its
// blocks are scheduled while the previous kernel of the stream drains; EPGPU_PDL=0 in the
// environment launches plainly instead.
// (off while a profiled step is launched, and for the one launch after an event record or wait of the
// step_fields hooks: an event between two kernels leaves no programmatic edge)
static thread_local bool g_pdl_suspended = false;
static thread_local bool g_pdl_skip_next = false;
static bool pdl_on() {
    static int on = -1;
    if (on < 0) {
        const char* e = getenv("EPGPU_PDL");
        on = (e && e[0] == '0') ? 0 : 1;
    }
    const bool skip = g_pdl_skip_next;
    g_pdl_skip_next = false;
    return on != 0 && !g_pdl_suspended && !skip;
}

// event record / wait of the step_fields hooks: external nodes when the stream is being captured (a
// plain record or wait inside a capture only orders the capture's own nodes)
static bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive;
}
static void hook_record(cudaEvent_t e, cudaStream_t s, bool internal) {
    if (!internal && capturing(s)) cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    else cudaEventRecord(e, s);
    g_pdl_skip_next = true;
}
static void hook_wait(cudaStream_t s, cudaEvent_t e, bool internal) {
    cudaStreamWaitEvent(s, e, (!internal && capturing(s)) ? cudaEventWaitExternal : 0);
    g_pdl_skip_next = true;
}

template <typename... K, typename... Args>
static void launch_pdl(void (*kern)(K...), int grid, int block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t c = {};
    c.gridDim = dim3((unsigned)grid);
    c.blockDim = dim3((unsigned)block);
    c.dynamicSmemBytes = 0;
    c.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = pdl_on() ? 1 : 0;
    c.attrs = at;
    c.numAttrs = 1;
    cudaLaunchKernelEx(&c, kern, static_cast<K>(args)...);
}

// step-start zeroing (km_zero) and the fused mUSL velocity + next-step cell scan (km_vmusl_scan)
static void launch_zero(const MixedCtx& X, cudaStream_t s) {
    const MCtx& A = *(const MCtx*)X.impl;
    const long long ng = (long long)(X.grid_zero_bytes / sizeof(float));
    const long long nz = (long long)(X.sort_zero_bytes / sizeof(int));
    const long long mx = (ng > nz ? ng : nz) / 4 + 1;
    const int nb = (int)std::min<long long>((mx + 255) / 256, 4LL * sm_count());
    launch_pdl(km_zero, nb > 0 ? nb : 1, 256, s, A, (float*)X.grid_zero, ng, (int*)X.sort_zero, nz, X.begin_step);
}

static void launch_vmusl_scan(const MCtx& A, bool musl, cudaStream_t s) {
    const int nt = scan_tiles(A.g.ncell);
    const int nv = musl ? (A.g.nnode + MSCAN2_BS - 1) / MSCAN2_BS : 0;
    launch_pdl(km_vmusl_scan, nt + nv, MSCAN2_BS, s, A, nt);
}


// ---------------------------------------------------------------------------
// import / export between the FP64 staging layout (P64: the reference's
// arrays as SoA) and the mixed state
// cell index of per-direction element indices: 2d ez + nz ex (tplgy.jl:49), 3d ez + nz ex + nz nx ey (tplgy.jl:82)
__device__ __forceinline__ int cell_of(const Geo& g, const int* e) {
    return g.dim == 2 ? e[1] + g.nel[1] * e[0] : e[2] + g.nel[2] * e[0] + g.nel[2] * g.nel[0] * e[1];
}
__device__ __forceinline__ void cell_dec(const Geo& g, int c, int* e) {
    if (g.dim == 2) {
        e[0] = c / g.nel[1];
        e[1] = c - e[0] * g.nel[1];
    } else {
        const int nzx = g.nel[2] * g.nel[0];
        e[1] = c / nzx;
        const int r = c - e[1] * nzx;
        e[0] = r / g.nel[2];
        e[2] = r - e[0] * g.nel[2];
    }
}

// symmetric storage of b: 2d (11, 22, 12), 3d Voigt (11, 22, 33, 23, 13, 12); Q.b is column-major D x D
__device__ __forceinline__ int sym_i(int D, int k) { return D == 2 ? (k == 2 ? 0 : k) : (k < 3 ? k : (k == 3 ? 1 : 0)); }
__device__ __forceinline__ int sym_j(int D, int k) { return D == 2 ? (k == 2 ? 1 : k) : (k < 3 ? k : (k == 5 ? 1 : 2)); }

// The staging fields in `mask` (EP_MPTS_* bits of the arrays they come from) into the mixed layout;
// the others keep their device values.
__global__ void km_import(MCtx A, P64 Q, uint64_t mask) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.P.np) return;
    const int D = A.g.dim, NS = D == 2 ? 3 : 6;
    const bool gimp = A.cf.basis == EP_BASIS_GIMPM;
    for (int d = 0; d < D; ++d) {
        if (mask & EP_MPTS_V) A.P.v[d][p] = (float)Q.v[d][p];
        if (gimp && (mask & EP_MPTS_L)) A.P.l[d][p] = (float)Q.l[d][p];
        if (gimp && (mask & EP_MPTS_L0)) A.P.l0[d][p] = (float)Q.l0[d][p];
    }
    if (mask & EP_MPTS_FIJ) {
        if (A.acc == 0) {
            for (int k = 0; k < D * D; ++k) A.P.Fd[k][p] = Q.F[k][p];
        } else {
            for (int k = 0; k < D * D; ++k) {
                const float h = (float)Q.F[k][p];
                A.P.Fh[k][p] = h;
                A.P.Fl[k][p] = (float)(Q.F[k][p] - (double)h);
            }
        }
    }
    if (mask & EP_MPTS_BIJ) {
        for (int k = 0; k < NS; ++k) {
            const int i = sym_i(D, k), j = sym_j(D, k);
            const double bs = 0.5 * (Q.b[i + D * j][p] + Q.b[j + D * i][p]);
            if (A.acc == 0) {
                A.P.bd[k][p] = bs;
            } else {
                const float h = (float)bs;
                A.P.bh[k][p] = h;
                A.P.bl[k][p] = (float)(bs - (double)h);
            }
        }
    }
    if (mask & EP_MPTS_EPII) {
        if (A.acc == 0) {
            A.P.ep1d[p] = Q.ep1[p];
        } else {
            const float h = (float)Q.ep1[p];
            A.P.ep1h[p] = h;
            A.P.ep1l[p] = (float)(Q.ep1[p] - (double)h);
        }
        A.P.ep2[p] = (float)Q.ep2[p];
    }
    if (A.cf.trsfr == EP_TRSFR_TPIC && (mask & EP_MPTS_DVIJ))
        for (int k = 0; k < D * D; ++k) A.P.dv[k][p] = (float)Q.dv[k][p];
    else if (A.cf.trsfr == EP_TRSFR_APIC && (mask & EP_MPTS_APIC_B))
        for (int k = 0; k < D * D; ++k) A.P.dv[k][p] = (float)Q.B[k][p];
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    if (mask & (fin ? EP_MPTS_TAU : EP_MPTS_SIG))
        for (int k = 0; k < NS; ++k) A.P.tau[k][p] = (float)(fin ? Q.tau[k][p] : Q.sig[k][p]);
    if (mask & EP_MPTS_DLAM) A.P.dlam[p] = (float)Q.dlam[p];
    if (mask & EP_MPTS_C0) A.P.c0[p] = (float)Q.c0[p];
    if (mask & EP_MPTS_CR) A.P.cr[p] = (float)Q.cr[p];
    if (mask & EP_MPTS_PHI) {
        A.P.tphi[p] = (float)Q.tphi[p];
        A.P.sphi[p] = (float)Q.sphi[p];
        A.P.cphi[p] = (float)Q.cphi[p];
    }
    // ρΩ: finite strain keeps ρΩ = ρ0Ω0 (deform.jl:1-24), so the mass is formed from the constants
    // (a resumed state's (ρ0/J)(J Ω0) could round to another FP32 value); infinitesimal strain
    // carries the current ρ Ω (deform.jl:25-44)
    if (mask & (fin ? (EP_MPTS_RHO0 | EP_MPTS_OMEGA0) : (EP_MPTS_RHO | EP_MPTS_OMEGA)))
        A.P.mp[p] = (float)(fin ? Q.rho0[p] * Q.Om0[p] : Q.rho[p] * Q.Om[p]);
    if (mask & EP_MPTS_OMEGA0) A.P.Om0[p] = (float)Q.Om0[p];
    if (mask & EP_MPTS_OMEGA) A.P.Om[p] = (float)Q.Om[p];
    if (mask & EP_MPTS_RHO) A.P.rho[p] = (float)Q.rho[p];
}

// Direct transfers (HostAoS) move a block's points [p0, p0 + n) of one host array at a time through
// shared memory in the host's own layout (k components per point), consecutive threads moving
// consecutive doubles, so that every warp access to the host link is one contiguous run; each thread
// then converts its own point from or to the shared copy.
constexpr int XH_BS = 256, XH_KMAX = 9;

__device__ __forceinline__ void xh_load(const double* __restrict__ host, int k, int p0, int n, double* sb) {
    __syncthreads();                                  // the previous field's readers are done with sb
    for (int i = threadIdx.x; i < k * n; i += XH_BS) sb[i] = host[(size_t)k * p0 + i];
    __syncthreads();
}

__device__ __forceinline__ void xh_store(double* host, int k, int p0, int n, const double* sb) {
    __syncthreads();                                  // every thread has put its point in sb
    for (int i = threadIdx.x; i < k * n; i += XH_BS) host[(size_t)k * p0 + i] = sb[i];
}

// Direct upload: the host arrays in `mask` into the mixed layout as km_import converts them, and the
// binning of km_bin0 from the host positions (which `mask` must include), in one pass over the points;
// the cell counts are added once per distinct cell of a warp.
// bin = 0: the arrays of the mask only (the positions, offsets and cell counts are left alone)
__device__ __forceinline__ void import_host_points(const MCtx& A, const HostAoS& H, uint64_t mask, int bin, int p0,
                                                   double* sb) {
    const int t = threadIdx.x, p = p0 + t;
    const int n = min(XH_BS, A.P.np - p0);
    const bool live = t < n;
    const int D = A.g.dim, NS = D == 2 ? 3 : 6, DD = D * D;
    if (bin) {
    const int cur = A.ctl->parity;
    xh_load(H.x, D, p0, n, sb);
    int c2 = -1;
    if (live) {
        bool fin = true;
        double x[3];
        for (int d = 0; d < D; ++d) {
            x[d] = sb[d + D * t];
            fin = fin && isfinite(x[d]);
        }
        if (fin) {
            int e[3];
            for (int d = 0; d < D; ++d) {
                e[d] = (int)fmin(fmax(floor((x[d] - A.g.x0[d]) / A.g.h[d]), 0.0), (double)(A.g.nel[d] - 1));
                A.P.dx[cur][d][p] = (float)(x[d] - A.g.ax[d][e[d]]);
            }
            c2 = cell_of(A.g, e);
        } else {
            set_err(A.ctl, EP_ERR_NONFINITE, p);
        }
        A.P.p2e_next[p] = c2;
        if (A.P.pcell[cur]) A.P.pcell[cur][p] = c2;
    }
    const unsigned mm = __match_any_sync(0xffffffffu, c2);
    if (c2 >= 0 && (t & 31) == __ffs(mm) - 1) atomicAdd(&A.S.count[cur][c2], __popc(mm));
    }
    if (mask & EP_MPTS_V) {
        xh_load(H.v, D, p0, n, sb);
        if (live)
            for (int d = 0; d < D; ++d) A.P.v[d][p] = (float)sb[d + D * t];
    }
    if (A.cf.basis == EP_BASIS_GIMPM && (mask & EP_MPTS_L)) {
        xh_load(H.l, D, p0, n, sb);
        if (live)
            for (int d = 0; d < D; ++d) A.P.l[d][p] = (float)sb[d + D * t];
    }
    if (mask & EP_MPTS_FIJ) {
        xh_load(H.F, DD, p0, n, sb);
        if (live)
            for (int k = 0; k < DD; ++k) {
                const double f = sb[k + DD * t];
                if (A.acc == 0) {
                    A.P.Fd[k][p] = f;
                } else {
                    const float h = (float)f;
                    A.P.Fh[k][p] = h;
                    A.P.Fl[k][p] = (float)(f - (double)h);
                }
            }
    }
    if (mask & EP_MPTS_BIJ) {
        xh_load(H.b, DD, p0, n, sb);
        if (live)
            for (int k = 0; k < NS; ++k) {
                const int i = sym_i(D, k), j = sym_j(D, k);
                const double bs = 0.5 * (sb[i + D * j + DD * t] + sb[j + D * i + DD * t]);
                if (A.acc == 0) {
                    A.P.bd[k][p] = bs;
                } else {
                    const float h = (float)bs;
                    A.P.bh[k][p] = h;
                    A.P.bl[k][p] = (float)(bs - (double)h);
                }
            }
    }
    if (mask & EP_MPTS_EPII) {
        xh_load(H.ep, 2, p0, n, sb);
        if (live) {
            const double e1 = sb[2 * t];
            if (A.acc == 0) {
                A.P.ep1d[p] = e1;
            } else {
                const float h = (float)e1;
                A.P.ep1h[p] = h;
                A.P.ep1l[p] = (float)(e1 - (double)h);
            }
            A.P.ep2[p] = (float)sb[2 * t + 1];
        }
    }
    if (A.cf.trsfr == EP_TRSFR_TPIC && (mask & EP_MPTS_DVIJ)) {
        xh_load(H.dv, DD, p0, n, sb);
        if (live)
            for (int k = 0; k < DD; ++k) A.P.dv[k][p] = (float)sb[k + DD * t];
    }
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    if (mask & (fin ? EP_MPTS_TAU : EP_MPTS_SIG)) {
        xh_load(fin ? H.tau : H.sig, NS, p0, n, sb);
        if (live)
            for (int k = 0; k < NS; ++k) A.P.tau[k][p] = (float)sb[k + NS * t];
    }
    if (mask & EP_MPTS_DLAM) {
        xh_load(H.dlam, 1, p0, n, sb);
        if (live) A.P.dlam[p] = (float)sb[t];
    }
}

// Direct download: the arrays in `mask` from the mixed layout as km_export forms them.
// par >= 0: the offset buffer of the positions (a download of x and v right after the G2P, while the
// rest of the step runs: the positions it wrote sit in the other parity until the step ends)
__device__ __forceinline__ void export_host_points(const MCtx& A, const HostAoS& H, uint64_t mask, int par, int p0,
                                                   double* sb) {
    const int t = threadIdx.x, p = p0 + t;
    const int n = min(XH_BS, A.P.np - p0);
    const bool live = t < n;
    const int cur = par >= 0 ? par : A.ctl->parity, D = A.g.dim, NS = D == 2 ? 3 : 6, DD = D * D;
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    if (mask & EP_MPTS_X) {
        // a point without a cell (non-finite position) keeps the host's value: a block holding one
        // reads its positions first
        const int c = live ? A.P.p2e_next[p] : 0;
        if (__syncthreads_or(live && c < 0)) xh_load(H.x, D, p0, n, sb);
        if (live && c >= 0) {
            int e[3];
            cell_dec(A.g, c, e);
            for (int d = 0; d < D; ++d) sb[d + D * t] = A.g.ax[d][e[d]] + (double)A.P.dx[cur][d][p];
        }
        xh_store(H.x, D, p0, n, sb);
    }
    if (mask & EP_MPTS_V) {
        __syncthreads();
        if (live)
            for (int d = 0; d < D; ++d) sb[d + D * t] = (double)A.P.v[d][p];
        xh_store(H.v, D, p0, n, sb);
    }
    if (A.cf.basis == EP_BASIS_GIMPM && (mask & EP_MPTS_L)) {
        __syncthreads();
        if (live)
            for (int d = 0; d < D; ++d) sb[d + D * t] = (double)A.P.l[d][p];
        xh_store(H.l, D, p0, n, sb);
    }
    double F[9], B[6];
    if (live && (mask & (EP_MPTS_FIJ | EP_MPTS_BIJ | (fin ? EP_MPTS_SIG : 0ull)))) {
        if (A.acc == 0) {
            for (int k = 0; k < DD; ++k) F[k] = A.P.Fd[k][p];
            for (int k = 0; k < NS; ++k) B[k] = A.P.bd[k][p];
        } else {
            for (int k = 0; k < DD; ++k) F[k] = (double)A.P.Fh[k][p] + (double)A.P.Fl[k][p];
            for (int k = 0; k < NS; ++k) B[k] = (double)A.P.bh[k][p] + (double)A.P.bl[k][p];
        }
    }
    if (mask & EP_MPTS_FIJ) {
        __syncthreads();
        if (live)
            for (int k = 0; k < DD; ++k) sb[k + DD * t] = F[k];
        xh_store(H.F, DD, p0, n, sb);
    }
    if (fin && (mask & EP_MPTS_BIJ)) {
        __syncthreads();
        if (live)
            for (int k = 0; k < NS; ++k) {
                const int i = sym_i(D, k), j = sym_j(D, k);
                sb[i + D * j + DD * t] = B[k];
                sb[j + D * i + DD * t] = B[k];
            }
        xh_store(H.b, DD, p0, n, sb);
    }
    if (mask & EP_MPTS_SIG) {
        __syncthreads();
        if (live) {
            double J = 1.0;
            if (fin)
                J = D == 2 ? F[0] * F[3] - F[2] * F[1]
                           : F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) +
                                 F[6] * (F[1] * F[5] - F[4] * F[2]);
            for (int k = 0; k < NS; ++k) sb[k + NS * t] = fin ? (double)A.P.tau[k][p] / J : (double)A.P.tau[k][p];
        }
        xh_store(H.sig, NS, p0, n, sb);
    }
    if (fin && (mask & EP_MPTS_TAU)) {
        __syncthreads();
        if (live)
            for (int k = 0; k < NS; ++k) sb[k + NS * t] = (double)A.P.tau[k][p];
        xh_store(H.tau, NS, p0, n, sb);
    }
    if (A.cf.trsfr == EP_TRSFR_TPIC && (mask & EP_MPTS_DVIJ)) {
        __syncthreads();
        if (live)
            for (int k = 0; k < DD; ++k) sb[k + DD * t] = (double)A.P.dv[k][p];
        xh_store(H.dv, DD, p0, n, sb);
    }
    if (mask & EP_MPTS_EPII) {
        __syncthreads();
        if (live) {
            const double e1 = A.acc == 0 ? A.P.ep1d[p] : (double)A.P.ep1h[p] + (double)A.P.ep1l[p];
            sb[2 * t] = e1;
            sb[2 * t + 1] = A.cf.nonloc ? (double)A.P.ep2[p] : e1;
        }
        xh_store(H.ep, 2, p0, n, sb);
    }
    if (mask & EP_MPTS_DLAM) {
        __syncthreads();
        if (live) sb[t] = (double)A.P.dlam[p];
        xh_store(H.dlam, 1, p0, n, sb);
    }
}

// XH_BS points per block and pass; a grid smaller than the point blocks (the transfers that overlap
// a running step) walks them, leaving the step's kernels room on the SMs
__global__ void __launch_bounds__(XH_BS) km_import_host(MCtx A, HostAoS H, uint64_t mask, int bin) {
    __shared__ double sb[XH_BS * XH_KMAX];
    for (int p0 = blockIdx.x * XH_BS; p0 < A.P.np; p0 += gridDim.x * XH_BS) {
        import_host_points(A, H, mask, bin, p0, sb);
        __syncthreads();
    }
}
__global__ void __launch_bounds__(XH_BS) km_export_host(MCtx A, HostAoS H, uint64_t mask, int par) {
    __shared__ double sb[XH_BS * XH_KMAX];
    for (int p0 = blockIdx.x * XH_BS; p0 < A.P.np; p0 += gridDim.x * XH_BS) {
        export_host_points(A, H, mask, par, p0, sb);
        __syncthreads();
    }
}

// initial cell, offsets and counts from the FP64 positions of the staging layout
__global__ void km_bin0(MCtx A, P64 Q) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = p < A.P.np;
    const int cur = A.ctl->parity, D = A.g.dim;
    int c2 = -1;
    if (live) {
        bool fin = true;
        double x[3];
        for (int d = 0; d < D; ++d) {
            x[d] = Q.x[d][p];
            fin = fin && isfinite(x[d]);
        }
        if (fin) {
            int e[3];
            for (int d = 0; d < D; ++d) {
                e[d] = (int)fmin(fmax(floor((x[d] - A.g.x0[d]) / A.g.h[d]), 0.0), (double)(A.g.nel[d] - 1));
                A.P.dx[cur][d][p] = (float)(x[d] - A.g.ax[d][e[d]]);
            }
            c2 = cell_of(A.g, e);
        } else {
            set_err(A.ctl, EP_ERR_NONFINITE, p);
        }
        A.P.p2e_next[p] = c2;
        if (A.P.pcell[cur]) A.P.pcell[cur][p] = c2;
    }
    // the counts once per distinct cell of the warp
    const unsigned mm = __match_any_sync(0xffffffffu, c2);
    if (c2 >= 0 && (threadIdx.x & 31) == __ffs(mm) - 1) atomicAdd(&A.S.count[cur][c2], __popc(mm));
}

__global__ void km_place0(MCtx A) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.P.np) return;
    place_next(A, p, A.ctl->parity);
}

// need_eps = 0: the log strain ϵ = ½ log b (FP64 eigen + log per point) is not formed; callers that
// do not read ϵ (masked downloads, conservation sums) skip that work.  mask: the staging arrays to
// write (EP_MPTS_* bits; the cell of each point always); a masked download moves only those.
__global__ void km_export(MCtx A, P64 Q, int need_eps, uint64_t mask) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.P.np) return;
    const int cur = A.ctl->parity, D = A.g.dim, NS = D == 2 ? 3 : 6;
    const int c = A.P.p2e_next[p];
    Q.p2e[p] = c;
    if (c >= 0 && (mask & EP_MPTS_X)) {
        int e[3];
        cell_dec(A.g, c, e);
        for (int d = 0; d < D; ++d) Q.x[d][p] = A.g.ax[d][e[d]] + (double)A.P.dx[cur][d][p];
    }
    for (int d = 0; d < D; ++d) {
        if (mask & EP_MPTS_V) Q.v[d][p] = (double)A.P.v[d][p];
        if (A.cf.basis == EP_BASIS_GIMPM && (mask & EP_MPTS_L)) Q.l[d][p] = (double)A.P.l[d][p];
    }
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    const uint64_t FDEP = EP_MPTS_FIJ | EP_MPTS_J | EP_MPTS_OMEGA | (fin ? (EP_MPTS_RHO | EP_MPTS_N | EP_MPTS_SIG) : 0ull);
    if (mask & (FDEP | EP_MPTS_BIJ | EP_MPTS_EIJ | EP_MPTS_TAU)) {
        double F[9], B[6];
        if (A.acc == 0) {
            for (int k = 0; k < D * D; ++k) F[k] = A.P.Fd[k][p];
            for (int k = 0; k < NS; ++k) B[k] = A.P.bd[k][p];
        } else {
            for (int k = 0; k < D * D; ++k) F[k] = (double)A.P.Fh[k][p] + (double)A.P.Fl[k][p];
            for (int k = 0; k < NS; ++k) B[k] = (double)A.P.bh[k][p] + (double)A.P.bl[k][p];
        }
        if (mask & EP_MPTS_FIJ)
            for (int k = 0; k < D * D; ++k) Q.F[k][p] = F[k];
        const double J = D == 2 ? F[0] * F[3] - F[2] * F[1]
                                : F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) +
                                      F[6] * (F[1] * F[5] - F[4] * F[2]);
        if (mask & EP_MPTS_J) Q.J[p] = J;
        // Ω = J Ω0 (deform.jl:18, 42); infinitesimal strain exports the volume the step carries and uses
        // (its FP32 J Ω0, which also sets the mass ρΩ), so that a download / upload round trip keeps it
        if (mask & EP_MPTS_OMEGA) Q.Om[p] = fin ? J * Q.Om0[p] : (double)A.P.Om[p];
        if (fin) {
            // finite strain: b, τ, σ = τ / J and ϵ = ½ log b (FP64, for output)
            if (mask & EP_MPTS_RHO) Q.rho[p] = Q.rho0[p] / J;
            if (mask & EP_MPTS_N) Q.n[p] = 1.0 - 1.0 / J * (1.0 - Q.n0[p]);
            for (int k = 0; k < NS; ++k) {
                if (mask & EP_MPTS_TAU) Q.tau[k][p] = (double)A.P.tau[k][p];
                if (mask & EP_MPTS_SIG) Q.sig[k][p] = (double)A.P.tau[k][p] / J;
            }
            if ((mask & EP_MPTS_BIJ) && D == 2) {
                Q.b[0][p] = B[0]; Q.b[3][p] = B[1]; Q.b[1][p] = B[2]; Q.b[2][p] = B[2];
            } else if (mask & EP_MPTS_BIJ) {
                for (int k = 0; k < 6; ++k) {
                    const int i = sym_i(3, k), j = sym_j(3, k);
                    Q.b[i + 3 * j][p] = B[k];
                    Q.b[j + 3 * i][p] = B[k];
                }
            }
            if (need_eps && D == 2) {
                double lam[2], V[4], L[2], R[4];
                eig_sym2(B[0], B[2], B[1], lam, V);
                L[0] = ep_log(lam[0]);
                L[1] = ep_log(lam[1]);
                vdvt<2>(V, L, R);
                for (int k = 0; k < 4; ++k) Q.eps[k][p] = 0.5 * R[k];
            } else if (need_eps) {
                double Bt[9], lam[3], V[9], L[3], R[9];
                for (int k = 0; k < 6; ++k) {
                    const int i = sym_i(3, k), j = sym_j(3, k);
                    Bt[i + 3 * j] = B[k];
                    Bt[j + 3 * i] = B[k];
                }
                eig_sym3(Bt, lam, V);
                for (int k = 0; k < 3; ++k) L[k] = ep_log(lam[k]);
                vdvt<3>(V, L, R);
                for (int k = 0; k < 9; ++k) Q.eps[k][p] = 0.5 * R[k];
            }
        }
    }
    if (!fin && (mask & EP_MPTS_SIG))
        for (int k = 0; k < NS; ++k) Q.sig[k][p] = (double)A.P.tau[k][p];
    if (A.cf.trsfr == EP_TRSFR_TPIC && (mask & EP_MPTS_DVIJ))
        for (int k = 0; k < D * D; ++k) Q.dv[k][p] = (double)A.P.dv[k][p];
    else if (A.cf.trsfr == EP_TRSFR_APIC && (mask & EP_MPTS_APIC_B))
        for (int k = 0; k < D * D; ++k) Q.B[k][p] = (double)A.P.dv[k][p];
    if (mask & EP_MPTS_EPII) {
        const double e1 = A.acc == 0 ? A.P.ep1d[p] : (double)A.P.ep1h[p] + (double)A.P.ep1l[p];
        Q.ep1[p] = e1;
        Q.ep2[p] = A.cf.nonloc ? (double)A.P.ep2[p] : e1;
    }
    if (mask & EP_MPTS_DLAM) Q.dlam[p] = (double)A.P.dlam[p];
}

// the nodal state of the last step: a, the damped force and (USL) v from its P2G fields by the
// step's own grid update (the fused G2P keeps them on chip), the mUSL momentum and velocity as stored
__global__ void km_export_nodes(MCtx A, N64 Q) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= A.g.nnode) return;
    const int D = A.g.dim;
    const float m = A.N.m[n];
    float a[3], v[3], f[3] = {0.f, 0.f, 0.f}, pn[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < D; ++d) {
        f[d] = A.N.f[d][n];
        pn[d] = A.N.p[d][n];
    }
    const int bc = A.g.bcw[n];
    grid_update(D, m, pn, f, bc, (float)A.ctl->dt, (float)A.cf.damping, a, v);
    const float mi = m != 0.f ? 1.f / m : 0.f;
    Q.m[n] = m;
    for (int d = 0; d < D; ++d) {
        // the mUSL velocity as vmusl_one forms it (the fused F-bar kernel keeps it on chip)
        const float vm = (m != 0.f && !((bc >> d) & 1)) ? A.N.pm[d][n] * mi : 0.f;
        Q.p[d][n] = A.cf.musl ? A.N.pm[d][n] : pn[d];
        Q.v[d][n] = A.cf.musl ? vm : v[d];
        Q.a[d][n] = a[d];
        Q.oobf[d][n] = f[d];
    }
    if (A.g.dim == 2) {
        const float4 q = A.N.vg4[n];
        Q.dJ[n] = 1.0 + (double)(A.cf.locking ? q.z * q.w : 0.f);
    } else {
        Q.dJ[n] = 1.0 + (double)A.N.dJn[n];
    }
}

// ===========================================================================
// 3d mixed step (infinitesimal strain: config 3's GIMP / TPIC / J2 and the DP
// variants).  Node id iz + nno_z ix + nno_z nno_x iy, cell ez + nz ex + nz nx ey
// (get_coords.jl:36-52, tplgy.jl:82); Voigt order (xx, yy, zz, yz, xz, xy).
__device__ __forceinline__ int node3(const Geo& g, const Axis4& ax, const Axis4& ay, const Axis4& az, int i, int j,
                                     int k) {
    return (az.base + k) + g.nno[2] * (ax.base + i) + g.nno[2] * g.nno[0] * (ay.base + j);
}

// FP32 J2 return in 3d (J2.jl:21-76 restated as in ep_scalar.h); the iteration stops at
// |f| <= max(1e-9, 2e-7 kappa), the resolution of an FP32 stress
__device__ __forceinline__ int j2f6(float* s, float ep2, float c0, float cr, float Hp, const float* D, float* g) {
    auto yield = [&](const float* v, float kap, float* n) {
        const float P = (v[0] + v[1] + v[2]) * (1.f / 3.f);
        float x[6];
        for (int i = 0; i < 3; ++i) x[i] = v[i] - P;
        for (int i = 3; i < 6; ++i) x[i] = v[i];
        const float j2 = 0.5f * (x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + 2.f * (x[3] * x[3] + x[4] * x[4] + x[5] * x[5]));
        const float xn = sqrtf(2.f * j2);
        for (int i = 0; i < 6; ++i) n[i] = x[i] / xn;
        return xn - kap;
    };
    float kap = fmaxf(cr, c0 + Hp * ep2), n[6];
    float f = yield(s, kap, n);
    if (!(f > 0.f)) return 0;
    float g0 = ep2;
    for (int it = 1; fabsf(f) > fmaxf(1.0e-9f, 2.0e-7f * kap) && it < 20; ++it) {
        float row[6];
        for (int j = 0; j < 6; ++j) {
            float a = 0.f;
            for (int i = 0; i < 6; ++i) a += n[i] * D[i + 6 * j];
            row[j] = a;
        }
        float den = 0.f;
        for (int j = 0; j < 6; ++j) den += row[j] * n[j];
        const float dl = f / den;
        for (int i = 0; i < 6; ++i) {
            float a = 0.f;
            for (int j = 0; j < 6; ++j) a += D[i + 6 * j] * n[j];
            s[i] -= dl * a;
        }
        g0 += dl;
        kap = fmaxf(cr, c0 + Hp * g0);
        f = yield(s, kap, n);
    }
    *g = g0;
    return 1;
}

// FP32 Drucker-Prager in 3d (DP.jl:33-98, outer cone DP.jl:19-21, ψ = 0); returns Δλ
__device__ __forceinline__ float dpf6(float* s, float ep2, float c0, float cr, float sphi, float cphi, float Kc,
                                      float Gc, float Hp, float* dep) {
    float coh = c0 + Hp * ep2;
    if (coh < cr) coh = cr;
    const float P = (s[0] + s[1] + s[2]) * (1.f / 3.f);
    float t[6];
    for (int i = 0; i < 3; ++i) t[i] = s[i] - P;
    for (int i = 3; i < 6; ++i) t[i] = s[i];
    const float tII = sqrtf(0.5f * (t[0] * t[0] + t[1] * t[1] + t[2] * t[2]) + t[3] * t[3] + t[4] * t[4] + t[5] * t[5]);
    const float sq3 = 1.7320508075688772f;
    const float eta = 6.f * sphi / (sq3 * (3.f + sphi)), xi = 6.f * coh * cphi / (sq3 * (3.f + sphi));
    const float sm = xi / eta, tP = xi - eta * sm;
    const float fs = tII + eta * P - xi;
    const float h = tII - tP - sqrtf(1.f + eta * eta) * (P - sm);
    float dl = 0.f;
    *dep = 0.f;
    if ((fs > 0.f && P < sm) || (h > 0.f && P >= sm)) {
        dl = fs / Gc;
        const float r = (xi - eta * P) / tII;
        for (int i = 0; i < 6; ++i) s[i] = t[i] * r + (i < 3 ? P : 0.f);
        *dep = dl * 0.57735026918962576f;
    }
    if (h <= 0.f && P >= sm) {
        dl = (P - sm) / Kc;
        const float Pn = sm - P, r = 0.f / tII;
        for (int i = 0; i < 6; ++i) s[i] = t[i] * r + (i < 3 ? Pn : 0.f);
        *dep = 1.41421356237309505f * dl / 3.f;
    }
    return dl;
}

struct PtW3 {
    int p, c, e[3];
    Axis4 a[3];
    float w[3][4], dw[3][4];
    float o[3];
};

template <int BASIS>
__device__ __forceinline__ bool point3(const MCtx& A, int cur, int k, int n, PtW3& W, bool& bad) {
    if (k >= n) {
        W.p = -1;
        W.c = -1;
        return false;
    }
    W.p = A.S.list[cur][k];
    W.c = A.S.cellof[cur][k];
    cell_dec(A.g, W.c, W.e);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        W.a[d] = axis4(A.g, d, W.e[d]);
        const float h = (float)A.g.h[d];
        W.o[d] = A.P.dx[cur][d][W.p];
        const float l = BASIS == EP_BASIS_GIMPM ? A.P.l[d][W.p] : 0.f;
        axis_w<BASIS>(W.a[d], W.o[d], h, 1.f / h, l, W.w[d], W.dw[d], bad);
    }
    return true;
}

// km_p2g_tile3: m, p, f in 3d (p2n.jl:58-102 std, 140-191 tpic).  TC cells per CTA; 16 lanes per
// cell, lane (qx, qy) owns the stencil column of 4 z-nodes
constexpr int TP3_STRIDE = 47;

// DET: each cell's node sums go to its 64 x 7 partials (m, p, f) for km_gather3 instead of FP32 atomics
template <int BASIS, int TC, bool DET = false>
__global__ void __launch_bounds__(16 * TC, 4) km_p2g_tile3(MCtx A) {
    constexpr int TH = 16 * TC;
    EP_ACTIVE(A.ctl);
    __shared__ float sp[TH * TP3_STRIDE];
    const int cur = A.ctl->parity;
    const int c0 = blockIdx.x * TC;
    if (c0 >= A.g.ncell) return;
    const int c1 = min(c0 + TC, A.g.ncell);
    const int* start = A.S.start[cur];
    const int b0 = start[c0], b1 = start[c1];
    if (b0 == b1) return;
    const int t = threadIdx.x;
    const int l16 = t & 15, qx = l16 & 3, qy = l16 >> 2, cl = c0 + (t >> 4);
    const bool cell_ok = cl < c1;
    const int pb = cell_ok ? start[cl] : 0, pe = cell_ok ? start[cl + 1] : 0;
    const float hx = (float)A.g.h[0], hy = (float)A.g.h[1], hz = (float)A.g.h[2];
    const float gz = (float)A.ctl->g[2];
    const bool tpic = A.cf.trsfr != EP_TRSFR_STD;   // v + G δ: TPIC's ∇v or APIC's Bᵢⱼ (D⁻¹ = I) in dv
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    float am[4], ap[3][4], af[3][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        am[j] = 0.f;
#pragma unroll
        for (int d = 0; d < 3; ++d) ap[d][j] = af[d][j] = 0.f;
    }
    bool bad = false;
    for (int ch = b0; ch < b1; ch += TH) {
        const int k = ch + t;
        if (k < b1) {
            const int p = A.S.list[cur][k], c = A.S.cellof[cur][k];
            int e[3];
            cell_dec(A.g, c, e);
            float* s = sp + t * TP3_STRIDE;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const Axis4 ax = axis4(A.g, d, e[d]);
                const float h = (float)A.g.h[d];
                const float o = A.P.dx[cur][d][p];
                const float l = BASIS == EP_BASIS_GIMPM ? A.P.l[d][p] : 0.f;
                axis_w<BASIS>(ax, o, h, 1.f / h, l, s + 8 * d, s + 8 * d + 4, bad);
                if (tpic) s[34 + d] = o;
            }
            const float sc = fin ? A.P.Om0[p] : A.P.Om[p];  // Ω σ = Ω0 τ (finite) or Ω σ
            s[24] = A.P.mp[p];
            s[25] = A.P.v[0][p];
            s[26] = A.P.v[1][p];
            s[27] = A.P.v[2][p];
#pragma unroll
            for (int v = 0; v < 6; ++v) s[28 + v] = sc * A.P.tau[v][p];
            if (tpic)
#pragma unroll
                for (int v = 0; v < 9; ++v) s[37 + v] = A.P.dv[v][p];
        }
        __syncthreads();
        const int lo = max(pb, ch), hi = min(pe, min(ch + TH, b1));
        for (int kk = lo; kk < hi; ++kk) {
            const float* s = sp + (kk - ch) * TP3_STRIDE;
            const float wxy = s[qx] * s[8 + qy], gx = s[4 + qx] * s[8 + qy], gy = s[qx] * s[12 + qy];
            const float ms = s[24];
            const float sxx = s[28], syy = s[29], szz = s[30], syz = s[31], sxz = s[32], sxy = s[33];
            float v0 = s[25], v1 = s[26], v2 = s[27], G[9], dlt0 = 0.f, dlt1 = 0.f, dz0 = 0.f;
            if (tpic) {
                // v + ∇v (x_n - x_p) with the previous step's ∇v (p2n.jl:157-158)
                dlt0 = (float)(qx - 1) * hx - s[34];
                dlt1 = (float)(qy - 1) * hy - s[35];
                dz0 = s[36];
#pragma unroll
                for (int v = 0; v < 9; ++v) G[v] = s[37 + v];
                v0 += G[0] * dlt0 + G[3] * dlt1;
                v1 += G[1] * dlt0 + G[4] * dlt1;
                v2 += G[2] * dlt0 + G[5] * dlt1;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float wz = s[16 + j], dwz = s[20 + j];
                const float N = wxy * wz, Nx = gx * wz, Ny = gy * wz, Nz = wxy * dwz;
                const float Nm = N * ms;
                am[j] += Nm;
                if (!tpic) {
                    ap[0][j] += Nm * s[25];
                    ap[1][j] += Nm * s[26];
                    ap[2][j] += Nm * s[27];
                } else {
                    const float dz = (float)(j - 1) * hz - dz0;
                    ap[0][j] += Nm * (v0 + G[6] * dz);
                    ap[1][j] += Nm * (v1 + G[7] * dz);
                    ap[2][j] += Nm * (v2 + G[8] * dz);
                }
                af[0][j] -= Nx * sxx + Ny * sxy + Nz * sxz;
                af[1][j] -= Nx * sxy + Ny * syy + Nz * syz;
                af[2][j] -= (Nx * sxz + Ny * syz + Nz * szz) - Nm * gz;
            }
        }
        __syncthreads();
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, c0);
    if (!cell_ok || pb == pe) return;
    if (DET) {
        // stencil slot (qx, qy, j) of the cell, all 64 written; km_gather3 adds them in a fixed order
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float* o = A.part + ((size_t)cl * 64 + l16 * 4 + j) * 7;
            o[0] = am[j];
            o[1] = ap[0][j]; o[2] = ap[1][j]; o[3] = ap[2][j];
            o[4] = af[0][j]; o[5] = af[1][j]; o[6] = af[2][j];
        }
        return;
    }
    int e[3];
    cell_dec(A.g, cl, e);
    const Axis4 ax = axis4(A.g, 0, e[0]), ay = axis4(A.g, 1, e[1]), az = axis4(A.g, 2, e[2]);
    if (ax.cls[qx] < 0 || ay.cls[qy] < 0) return;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (az.cls[j] < 0) continue;
        const int n = node3(A.g, ax, ay, az, qx, qy, j);
        atomicAdd(&A.N.m[n], am[j]);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            atomicAdd(&A.N.p[d][n], ap[d][j]);
            atomicAdd(&A.N.f[d][n], af[d][j]);
        }
    }
}

// Deterministic scatters in 3d, the tile staging of km_p2g_tile3: the mUSL momentum (KIND 1: m v per
// point, augm.jl:13-25) and Σ N m δJ (KIND 2: the per-point value left in ptmp by km_fbar_seg3,
// volumetric.jl:1-11), each cell's points summed in list (point id) order into its 64 x NQ partials
template <int BASIS, int TC, int KIND>
__global__ void __launch_bounds__(16 * TC) km_aux_tile3(MCtx A) {
    constexpr int TH = 16 * TC, NQ = KIND == 1 ? 3 : 1, ST = 17;
    EP_ACTIVE(A.ctl);
    __shared__ float sp[TH * ST];
    const int cur = A.ctl->parity;
    const int c0 = blockIdx.x * TC;
    if (c0 >= A.g.ncell) return;
    const int c1 = min(c0 + TC, A.g.ncell);
    const int* start = A.S.start[cur];
    const int b0 = start[c0], b1 = start[c1];
    if (b0 == b1) return;
    const int t = threadIdx.x;
    const int l16 = t & 15, qx = l16 & 3, qy = l16 >> 2, cl = c0 + (t >> 4);
    const bool cell_ok = cl < c1;
    const int pb = cell_ok ? start[cl] : 0, pe = cell_ok ? start[cl + 1] : 0;
    float acc[4][NQ];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int v = 0; v < NQ; ++v) acc[j][v] = 0.f;
    bool bad = false;
    for (int ch = b0; ch < b1; ch += TH) {
        const int k = ch + t;
        if (k < b1) {
            const int p = A.S.list[cur][k], c = A.S.cellof[cur][k];
            int e[3];
            cell_dec(A.g, c, e);
            float* s = sp + t * ST;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const Axis4 ax = axis4(A.g, d, e[d]);
                const float h = (float)A.g.h[d];
                const float l = BASIS == EP_BASIS_GIMPM ? A.P.l[d][p] : 0.f;
                float dw[4];
                axis_w<BASIS>(ax, A.P.dx[cur][d][p], h, 1.f / h, l, s + 4 * d, dw, bad);
            }
            if (KIND == 1) {
                const float mp = A.P.mp[p];
#pragma unroll
                for (int d = 0; d < 3; ++d) s[12 + d] = mp * A.P.v[d][p];
            } else {
                s[12] = A.ptmp[p];
            }
        }
        __syncthreads();
        const int lo = max(pb, ch), hi = min(pe, min(ch + TH, b1));
        for (int kk = lo; kk < hi; ++kk) {
            const float* s = sp + (kk - ch) * ST;
            const float wxy = s[qx] * s[4 + qy];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float N = wxy * s[8 + j];
#pragma unroll
                for (int v = 0; v < NQ; ++v) acc[j][v] += N * s[12 + v];
            }
        }
        __syncthreads();
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, c0);
    if (!cell_ok || pb == pe) return;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int v = 0; v < NQ; ++v) A.part[((size_t)cl * 64 + l16 * 4 + j) * NQ + v] = acc[j][v];
}

// node sums of the 3d per-cell partials: node (iy, ix, iz) is slot (qx, qy, r) of the cell
// (ey, ex, ez) = (iy + 1 - qy, ix + 1 - qx, iz + 1 - r); cells visited in that fixed order
template <int NQ>
__global__ void km_gather3(MCtx A, float* o0, float* o1, float* o2, float* o3, float* o4, float* o5, float* o6) {
    EP_ACTIVE(A.ctl);
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= A.g.nnode) return;
    const int cur = A.ctl->parity;
    const int nz = A.g.nno[2], nzx = nz * A.g.nno[0];
    const int iy = n / nzx, rem = n - iy * nzx, ix = rem / nz, iz = rem - ix * nz;
    const int ncz = A.g.nel[2], nczx = ncz * A.g.nel[0];
    const int* start = A.S.start[cur];
    float acc[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) acc[v] = 0.f;
#pragma unroll 1
    for (int qy = 0; qy < 4; ++qy) {
        const int ey = iy + 1 - qy;
        if (ey < 0 || ey >= A.g.nel[1]) continue;
#pragma unroll 1
        for (int qx = 0; qx < 4; ++qx) {
            const int ex = ix + 1 - qx;
            if (ex < 0 || ex >= A.g.nel[0]) continue;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int ez = iz + 1 - r;
                if (ez < 0 || ez >= ncz) continue;
                const int c = ez + ncz * ex + nczx * ey;
                if (start[c] == start[c + 1]) continue;
                const float* pp = A.part + ((size_t)c * 64 + (qx + 4 * qy) * 4 + r) * NQ;
#pragma unroll
                for (int v = 0; v < NQ; ++v) acc[v] += pp[v];
            }
        }
    }
    float* outs[7] = {o0, o1, o2, o3, o4, o5, o6};
#pragma unroll
    for (int v = 0; v < NQ; ++v) outs[v][n] = acc[v];
}

// km_g2p_seg3: PIC/FLIP (n2p.jl:14-40), new cell + offset, vmax, next-cell counts and the
// mUSL momentum P2G (augm.jl:13-25) in 3d, one lane per point
// DET: the momentum P2G is left to km_aux_tile3<.., 1> (no FP32 atomics); AP: APIC's Bᵢⱼ is formed
// (a separate instantiation, so that the other transfers keep their register budget)
template <int BASIS, bool DET = false, bool AP = false>
__global__ void __launch_bounds__(256) km_g2p_seg3(MCtx A) {
    EP_ACTIVE(A.ctl);
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int n = A.S.start[cur][A.g.ncell];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = false;
    PtW3 W;
    const bool live = point3<BASIS>(A, cur, k, n, W, bad);
    const Seg S = seg_of(W.c);
    const float dtf = (float)A.ctl->dt, Cpf = (float)A.cf.Cpf;
    unsigned vm[3] = {0u, 0u, 0u};
    float v[3] = {0.f, 0.f, 0.f}, mp = 0.f;
    int c2 = -1;
    if (live) {
        float vp[3] = {0.f, 0.f, 0.f}, af[3] = {0.f, 0.f, 0.f};
#pragma unroll 1
        for (int j = 0; j < 4; ++j) {
            if (W.a[1].cls[j] < 0) continue;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (W.a[0].cls[i] < 0) continue;
                const float wxy = W.w[0][i] * W.w[1][j];
#pragma unroll
                for (int kz = 0; kz < 4; ++kz) {
                    if (W.a[2].cls[kz] < 0) continue;
                    const int nd = node3(A.g, W.a[0], W.a[1], W.a[2], i, j, kz);
                    const float N = wxy * W.w[2][kz];
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        vp[d] += N * __ldg(&A.N.v[d][nd]);
                        af[d] += N * __ldg(&A.N.a[d][nd]);
                    }
                }
            }
        }
        const int p = W.p;
        if (AP) {
            // Bᵢⱼ = Σ N v_n δᵀ, δ = node - point at the step start (Bij.jl:14-26)
            float B[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
            for (int j = 0; j < 4; ++j) {
                if (W.a[1].cls[j] < 0) continue;
                const float dly = (float)(j - 1) * (float)A.g.h[1] - W.o[1];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    if (W.a[0].cls[i] < 0) continue;
                    const float dlx = (float)(i - 1) * (float)A.g.h[0] - W.o[0];
                    const float wxy = W.w[0][i] * W.w[1][j];
#pragma unroll
                    for (int kz = 0; kz < 4; ++kz) {
                        if (W.a[2].cls[kz] < 0) continue;
                        const int nd = node3(A.g, W.a[0], W.a[1], W.a[2], i, j, kz);
                        const float N = wxy * W.w[2][kz];
                        const float dl[3] = {dlx, dly, (float)(kz - 1) * (float)A.g.h[2] - W.o[2]};
                        float vn[3];
#pragma unroll
                        for (int d = 0; d < 3; ++d) vn[d] = __ldg(&A.N.v[d][nd]);
#pragma unroll
                        for (int b = 0; b < 3; ++b)
#pragma unroll
                            for (int a = 0; a < 3; ++a) B[a + 3 * b] += N * (vn[a] * dl[b]);
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < 9; ++k) A.P.dv[k][p] = B[k];
        }
        int e2[3];
        float o2[3];
        bool fin = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            v[d] = Cpf * (A.P.v[d][p] + dtf * af[d]) + (1.f - Cpf) * vp[d];
            A.P.v[d][p] = v[d];
            vm[d] = __float_as_uint(fabsf(v[d]));
            const float o = W.o[d] + dtf * vp[d];
            fin = fin && isfinite(o);
            if (isfinite(o)) recell(A.g, d, W.e[d], o, 1.f / (float)A.g.h[d], e2[d], o2[d]);
        }
        if (fin) {
            c2 = cell_of(A.g, e2);
#pragma unroll
            for (int d = 0; d < 3; ++d) A.P.dx[nxt][d][p] = o2[d];
        } else {
            set_err(A.ctl, EP_ERR_NONFINITE, p);
        }
        A.P.p2e_next[p] = c2;
        if (A.P.pcell[nxt]) A.P.pcell[nxt][p] = c2;
        mp = A.P.mp[p];
    }
    {
        const unsigned mm = __match_any_sync(0xffffffffu, c2);
        if (c2 >= 0 && S.lane == __ffs(mm) - 1) atomicAdd(&A.S.count[nxt][c2], __popc(mm));
    }
    if (!DET && A.cf.musl) {
#pragma unroll 1
        for (int j = 0; j < 4; ++j)
#pragma unroll 1
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int kz = 0; kz < 4; ++kz) {
                    const float Nm = live ? W.w[0][i] * W.w[1][j] * W.w[2][kz] * mp : 0.f;
                    const float s0 = seg_sum(Nm * v[0], S), s1 = seg_sum(Nm * v[1], S), s2 = seg_sum(Nm * v[2], S);
                    if (S.head && live && W.a[0].cls[i] >= 0 && W.a[1].cls[j] >= 0 && W.a[2].cls[kz] >= 0) {
                        const int nd = node3(A.g, W.a[0], W.a[1], W.a[2], i, j, kz);
                        atomicAdd(&A.N.pm[0][nd], s0);
                        atomicAdd(&A.N.pm[1][nd], s1);
                        atomicAdd(&A.N.pm[2][nd], s2);
                    }
                }
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, W.c);
#pragma unroll
    for (int d = 0; d < 3; ++d) vm[d] = __reduce_max_sync(0xffffffffu, vm[d]);
    if (S.lane == 0)
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (vm[d])
                atomicMax(&A.ctl->vmax_bits[d], (unsigned long long)__double_as_longlong((double)__uint_as_float(vm[d])));
}

// ∇v of a point in 3d: g[i + 3 j] = Σ_n ∂N/∂x_j v_i(n) (deform.jl:9-10), optionally a = Σ N δJ_n
__device__ __forceinline__ void grad3(const MCtx& A, const PtW3& W, float* const* vn, float* g, bool lock, float* a) {
#pragma unroll
    for (int i = 0; i < 9; ++i) g[i] = 0.f;
    float s = 0.f;
#pragma unroll 1
    for (int j = 0; j < 4; ++j) {
        if (W.a[1].cls[j] < 0) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (W.a[0].cls[i] < 0) continue;
#pragma unroll
            for (int kz = 0; kz < 4; ++kz) {
                if (W.a[2].cls[kz] < 0) continue;
                const int nd = node3(A.g, W.a[0], W.a[1], W.a[2], i, j, kz);
                const float dN[3] = {W.dw[0][i] * W.w[1][j] * W.w[2][kz], W.w[0][i] * W.dw[1][j] * W.w[2][kz],
                                     W.w[0][i] * W.w[1][j] * W.dw[2][kz]};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float vc = __ldg(&vn[c][nd]);
#pragma unroll
                    for (int d = 0; d < 3; ++d) g[c + 3 * d] += dN[d] * vc;
                }
                if (lock) s += W.w[0][i] * W.w[1][j] * W.w[2][kz] * __ldg(&A.N.dJn[nd]);
            }
        }
    }
    *a = s;
}

// km_fbar_seg3: δJ = det(I + dt ∇v) - 1 and Σ N m δJ (deform.jl:9-18, volumetric.jl:1-11) in 3d
// DET: the point's m δJ goes to ptmp for km_aux_tile3<.., 2> (no FP32 atomics)
template <int BASIS, bool DET = false>
__global__ void __launch_bounds__(256) km_fbar_seg3(MCtx A) {
    EP_ACTIVE(A.ctl);
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int n = A.S.start[cur][A.g.ncell];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = false;
    PtW3 W;
    const bool live = point3<BASIS>(A, cur, k, n, W, bad);
    const Seg S = seg_of(W.c);
    const float dtf = (float)A.ctl->dt;
    float* const* vn = A.cf.musl ? A.N.vm : A.N.v;
    const bool fin = A.cf.deform == EP_DEFORM_FINITE;
    float mdj = 0.f;
    if (live) {
        float g[9], unused;
        grad3(A, W, vn, g, false, &unused);
        float D[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) D[i] = dtf * g[i];
        const float dJ = det1p_m1(D);
        mdj = A.P.mp[W.p] * (fin ? dJ : dJ * (2.f + dJ));
    }
    place_next_warp(A, live ? W.p : -1, live ? A.P.p2e_next[W.p] : -1, nxt, S.lane);
    if (DET) {
        if (live) A.ptmp[W.p] = mdj;
    } else {
#pragma unroll 1
        for (int j = 0; j < 4; ++j)
#pragma unroll 1
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int kz = 0; kz < 4; ++kz) {
                    const float v = seg_sum(live ? W.w[0][i] * W.w[1][j] * W.w[2][kz] * mdj : 0.f, S);
                    if (S.head && live && W.a[0].cls[i] >= 0 && W.a[1].cls[j] >= 0 && W.a[2].cls[kz] >= 0)
                        atomicAdd(&A.N.dJacc[node3(A.g, W.a[0], W.a[1], W.a[2], i, j, kz)], v);
                }
    }
    if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, W.c);
}

// km_nonlocal3: the nonlocal averaging of km_nonlocal in 3d (the FP64 step's k_nonlocal64<3>):
// candidates from the cells within ±nnel of p's step-start cell, in ascending id order, the
// distance in the first two coordinates (x, y) as the reference forms it (nonlocal.jl:27-28)
template <int ACC>
__global__ void __launch_bounds__(32) km_nonlocal3(MCtx A) {
    EP_ACTIVE(A.ctl);
    __shared__ int qs[NLM_CAP];
    __shared__ float om[NLM_CAP];
    const int p = blockIdx.x, lane = threadIdx.x;
    if (p >= A.P.np) return;
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int cp = A.P.pcell[cur][p], cn = A.P.pcell[nxt][p];
    if (A.P.dlam[p] == 0.f || cp < 0 || cn < 0) {
        if (lane == 0) A.P.ep2[p] = 0.f;
        return;
    }
    int e[3];
    cell_dec(A.g, cp, e);
    int lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        lo[d] = max(e[d] - A.g.nnel[d], 0);
        hi[d] = min(e[d] + A.g.nnel[d], A.g.nel[d] - 1);
    }
    const int nz = A.g.nel[2], nzx = A.g.nel[2] * A.g.nel[0];
    const int* start = A.S.start[cur];
    const int* list = A.S.list[cur];
    // each (y, x) column's z-run of cells is one contiguous slice of the list
    int L = 0;
    for (int k = lo[1]; k <= hi[1]; ++k)
        for (int a = lo[0]; a <= hi[0]; ++a) L += start[hi[2] + nz * a + nzx * k + 1] - start[lo[2] + nz * a + nzx * k];
    const double ls = A.cf.ls;
    int en[3];
    cell_dec(A.g, cn, en);
    const double xp0 = A.g.ax[0][en[0]] + (double)A.P.dx[nxt][0][p];
    const double xp1 = A.g.ax[1][en[1]] + (double)A.P.dx[nxt][1][p];
    auto omega = [&](int q) {
        int eq[3];
        cell_dec(A.g, A.P.pcell[nxt][q], eq);
        const double xi = xp0 - (A.g.ax[0][eq[0]] + (double)A.P.dx[nxt][0][q]);
        const double et = xp1 - (A.g.ax[1][eq[1]] + (double)A.P.dx[nxt][1][q]);
        const float r = (float)(sqrt(xi * xi + et * et) / ls);
        return r * expf(-(r * r));
    };
    if (L <= NLM_CAP) {
        int pos = 0;
        for (int k = lo[1]; k <= hi[1]; ++k)
            for (int a = lo[0]; a <= hi[0]; ++a) {
                const int b = start[lo[2] + nz * a + nzx * k], n = start[hi[2] + nz * a + nzx * k + 1] - b;
                for (int t = lane; t < n; t += 32) qs[pos + t] = list[b + t];
                pos += n;
            }
        int P2 = 32;
        while (P2 < L) P2 <<= 1;
        for (int t = L + lane; t < P2; t += 32) qs[t] = INT_MAX;
        __syncwarp();
        for (int kk = 2; kk <= P2; kk <<= 1)
            for (int j = kk >> 1; j > 0; j >>= 1) {
                for (int t = lane; t < P2; t += 32) {
                    const int q = t ^ j;
                    if (q > t) {
                        const int x = qs[t], c = qs[q];
                        const bool asc = (t & kk) == 0;
                        if ((x > c) == asc) {
                            qs[t] = c;
                            qs[q] = x;
                        }
                    }
                }
                __syncwarp();
            }
        for (int t = lane; t < L; t += 32) om[t] = omega(qs[t]);
        __syncwarp();
        if (lane == 0) {
            float W = 0.f;
            for (int t = 0; t < L; ++t) {
                const int q = qs[t];
                if (q >= p) break;
                if (A.P.dlam[q] != 0.f) W += om[t];
            }
            for (int t = 0; t < L; ++t) {
                const int q = qs[t];
                if (q < p && A.P.dlam[q] != 0.f) continue;
                W += om[t];
            }
            float sum = 0.f;
            if (!(W > 1e-16f)) {
                sum = ep1_of<ACC>(A, p);
            } else {
                for (int t = 0; t < L; ++t) {
                    const int q = qs[t];
                    if (q < p && A.P.dlam[q] != 0.f) continue;
                    sum += (om[t] / W) * ep1_of<ACC>(A, q);
                }
            }
            A.P.ep2[p] = sum;
        }
        return;
    }
    // more candidates than the shared buffer holds: ascending order by repeated minimum selection
    if (lane != 0) return;
    float W = 0.f;
    for (int pass = 0; pass < 3; ++pass) {
        float sum = 0.f;
        int last = -1;
        if (pass == 2 && !(W > 1e-16f)) {
            A.P.ep2[p] = ep1_of<ACC>(A, p);
            return;
        }
        while (true) {
            int best = INT_MAX;
            for (int k = lo[1]; k <= hi[1]; ++k)
                for (int a = lo[0]; a <= hi[0]; ++a)
                    for (int t = start[lo[2] + nz * a + nzx * k]; t < start[hi[2] + nz * a + nzx * k + 1]; ++t) {
                        const int q = list[t];
                        if (q > last && q < best) best = q;
                    }
            if (best == INT_MAX) break;
            last = best;
            const int q = best;
            const bool plq = A.P.dlam[q] != 0.f;
            if (pass == 0 && !(q < p && plq)) continue;
            if (pass >= 1 && (q < p && plq)) continue;
            const float w = omega(q);
            if (pass < 2) W += w;
            else sum += (w / W) * ep1_of<ACC>(A, q);
        }
        if (pass == 2) A.P.ep2[p] = sum;
    }
}

// ---------------------------------------------------------------------------
// 3d finite strain.  b_e is kept as its deviation M = b_e - I (formed exactly from the FP64 value
// or the hi + lo pair), so the eigenvalues mu of M carry the strain to the relative precision of
// the arithmetic: ε_i = ½ log(1 + mu_i) (elast.jl:51-52).  FP32: cyclic Jacobi on M (Golub & Van
// Loan, Matrix Computations, sym.Schur2 and the cyclic Jacobi method, the algorithm of ep_scalar.h
// eig_sym3); FP64 storage ("mixed"): eig_sym3 itself on M in FP64.

// sym index k (Voigt xx, yy, zz, yz, xz, xy) -> (i, j)
__host__ __device__ constexpr int vi3(int k) { return k < 3 ? k : (k == 3 ? 1 : 0); }
__host__ __device__ constexpr int vj3(int k) { return k < 3 ? k : (k == 5 ? 1 : 2); }

// Voigt components of V diag(d) V'
template <typename R>
__device__ __forceinline__ void vdv3(const R (&V)[3][3], const R* d, R* out) {
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int i = vi3(k), j = vj3(k);
        out[k] = V[i][0] * V[j][0] * d[0] + V[i][1] * V[j][1] * d[1] + V[i][2] * V[j][2] * d[2];
    }
}

// b_e = V diag(exp 2ε) V' (DP.jl:63-66) of returned principal log strains, into the point's
// accumulated storage as I + V diag(expm1 2ε) V'
template <int ACC, typename R>
__device__ __forceinline__ void rebuild_b3(const MCtx& A, int p, const R (&V)[3][3], const R* eps) {
    R d[3], dev[6];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (ACC == 0) d[i] = (R)(ep_exp(2.0 * (double)eps[i]) - 1.0);
        else d[i] = (R)expm1f(2.f * (float)eps[i]);
    }
    vdv3<R>(V, d, dev);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        if (ACC == 0) {
            A.P.bd[k][p] = (k < 3 ? 1.0 : 0.0) + (double)dev[k];
        } else {
            float h, l;
            if (k < 3) {
                df_one_plus((float)dev[k], h, l);
            } else {
                h = (float)dev[k];
                l = 0.f;
            }
            A.P.bh[k][p] = h;
            A.P.bl[k][p] = l;
        }
    }
}

// b <- ΔF b ΔF' = b + (T + T' + T D'), T = D b (elast.jl:49), then the trial principal log
// strains ε (elast.jl:51-52) and the eigenvectors V of b (columns)
template <int ACC, typename R>
__device__ __forceinline__ void trial_log_strain3(const MCtx& A, int p, const float* D, R (&V)[3][3], R* eps) {
    float bf[3][3];
    double Bd[6];
    float Bh[6], Bl[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        if (ACC == 0) {
            Bd[k] = A.P.bd[k][p];
            bf[vi3(k)][vj3(k)] = bf[vj3(k)][vi3(k)] = (float)Bd[k];
        } else {
            Bh[k] = A.P.bh[k][p];
            Bl[k] = A.P.bl[k][p];
            bf[vi3(k)][vj3(k)] = bf[vj3(k)][vi3(k)] = Bh[k];
        }
    }
    float T[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) T[i][j] = D[i] * bf[0][j] + D[i + 3] * bf[1][j] + D[i + 6] * bf[2][j];
    R M[3][3];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int i = vi3(k), j = vj3(k);
        const float inc = T[i][j] + T[j][i] + (T[i][0] * D[j] + T[i][1] * D[j + 3] + T[i][2] * D[j + 6]);
        R m;
        if (ACC == 0) {
            Bd[k] += (double)inc;
            A.P.bd[k][p] = Bd[k];
            m = (R)(k < 3 ? Bd[k] - 1.0 : Bd[k]);
        } else {
            df_add(Bh[k], Bl[k], inc);
            A.P.bh[k][p] = Bh[k];
            A.P.bl[k][p] = Bl[k];
            m = (R)(k < 3 ? (Bh[k] - 1.f) + Bl[k] : Bh[k] + Bl[k]);
        }
        M[i][j] = M[j][i] = m;
    }
    if (ACC == 0) {
        double a[9], lam[3], W[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) a[i + 3 * j] = (double)M[i][j];
        eig_sym3(a, lam, W);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            eps[i] = (R)(0.5 * ep_log(1.0 + lam[i]));
#pragma unroll
            for (int j = 0; j < 3; ++j) V[i][j] = (R)W[i + 3 * j];
        }
    } else {
        float a[3][3], v[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) a[i][j] = (float)M[i][j];
        eig3f(a, v);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            eps[i] = (R)(0.5f * log1pf(a[i][i]));
#pragma unroll
            for (int j = 0; j < 3; ++j) V[i][j] = (R)v[i][j];
        }
    }
}

// eigenvalues and eigenvectors of the strain tensor of an engineering Voigt strain
// (xx, yy, zz, 2yz, 2xz, 2xy): tensor_from_voigt(ε, ½) of DP.jl:63-64, FP32 or FP64
template <typename R>
__device__ __forceinline__ void eig_voigt3(const float* ev, R (&V)[3][3], R* lam) {
    if (sizeof(R) == 8) {
        double a[9], l[3], W[9];
        a[0] = ev[0]; a[4] = ev[1]; a[8] = ev[2];
        a[5] = a[7] = 0.5 * (double)ev[3];
        a[2] = a[6] = 0.5 * (double)ev[4];
        a[1] = a[3] = 0.5 * (double)ev[5];
        eig_sym3(a, l, W);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            lam[i] = (R)l[i];
#pragma unroll
            for (int j = 0; j < 3; ++j) V[i][j] = (R)W[i + 3 * j];
        }
    } else {
        float a[3][3], v[3][3];
        a[0][0] = ev[0]; a[1][1] = ev[1]; a[2][2] = ev[2];
        a[1][2] = a[2][1] = 0.5f * ev[3];
        a[0][2] = a[2][0] = 0.5f * ev[4];
        a[0][1] = a[1][0] = 0.5f * ev[5];
        eig3f(a, v);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            lam[i] = (R)a[i][i];
#pragma unroll
            for (int j = 0; j < 3; ++j) V[i][j] = (R)v[i][j];
        }
    }
}

// 3d features of a finite-strain DP trial (ep_rmap.h layout, x7 = 1) from its principal log
// strains: sorted descending, V's columns with them; aux = V (column-major), s, c
__device__ __forceinline__ bool rm_features3(const float* eps_in, const float (&Vin)[3][3], float coh, float tphi,
                                             float Gc, float l2g, float* x, float* aux) {
    float e[3] = {eps_in[0], eps_in[1], eps_in[2]};
    int o[3] = {0, 1, 2};
    auto cswap = [&](int a, int b) {
        if (e[a] < e[b]) {
            const float t = e[a]; e[a] = e[b]; e[b] = t;
            const int q = o[a]; o[a] = o[b]; o[b] = q;
        }
    };
    cswap(0, 1);
    cswap(1, 2);
    cswap(0, 1);
    const float s = coh / (2.f * Gc);
    const float e1 = e[0] / s, e2 = e[1] / s, e3 = e[2] / s;
    const float tr = e1 + e2 + e3;
    const float t1 = l2g * tr + e1, t2 = l2g * tr + e2, t3 = l2g * tr + e3;
    const float P = (t1 + t2 + t3) * (1.f / 3.f);
    const float d1 = t1 - P, d2 = t2 - P, d3 = t3 - P;
    const float tII = sqrtf(0.5f * (d1 * d1 + d2 * d2 + d3 * d3));
    const float rr = rsqrtf(1.f + tphi * tphi), sphi = tphi * rr, cphi = rr;
    const float eta = 6.f * sphi / (1.7320508075688772f * (3.f + sphi));
    const float xi = 6.f * cphi / (1.7320508075688772f * (3.f + sphi));
    const float fs = tII + eta * P - xi;
    x[0] = e1; x[1] = e2; x[2] = e3; x[3] = coh * (float)(1.0 / RM_CREF);
    x[4] = tphi; x[5] = 0.f; x[6] = fmaxf(fs, 0.f); x[7] = 1.f;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int oc = o[c];
            aux[i + 3 * c] = oc == 0 ? Vin[i][0] : (oc == 1 ? Vin[i][1] : Vin[i][2]);
        }
    aux[9] = s;
    aux[10] = coh;
    aux[11] = 0.f;
    return (fs > 0.f && P < xi / eta) || P >= xi / eta;
}

// km_cons3: F-bar, F, the elastic predictor -- finite (log strain / Kirchhoff, elast.jl:45-56) or
// infinitesimal (elast.jl:69-80) -- and the J2 / DP returns in 3d, one lane per sorted point.
// Finite strain works in the principal frame of the trial b_e: with the isotropic stiffness the
// trial Kirchhoff stress, both returns and b_e = exp(2 Del \ τ) (DP.jl:63-66) are coaxial with it.
// With the learned return map a trial-yielding DP point is handed to the network as in 2d.
template <int BASIS, int ACC, bool FIN, bool ITER = false>
__global__ void __launch_bounds__(256, 3) km_cons3(MCtx A, int plastic_phase) {
    using R = typename std::conditional<ACC == 0, double, float>::type;
    EP_ACTIVE(A.ctl);
    const int cur = A.ctl->parity, nxt = cur ^ 1;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int nplastic = 0;
    const int n = A.S.start[cur][A.g.ncell];
    bool emit = false;
    float fx[RM_NX], fy[RM_NY], fa[12];
    int fp = 0;
    if (k < n) {
        bool bad = false;
        PtW3 W;
        point3<BASIS>(A, cur, k, n, W, bad);
        const int p = W.p;
        fp = p;
        const float dtf = (float)A.ctl->dt;
        const bool lock = A.cf.locking;
        float g[9], a = 0.f;
        grad3(A, W, A.cf.musl ? A.N.vm : A.N.v, g, lock, &a);
        float D[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) D[i] = dtf * g[i];
        if (A.cf.trsfr == EP_TRSFR_TPIC)
#pragma unroll
            for (int i = 0; i < 9; ++i) A.P.dv[i][p] = g[i];
        // F <- ΔF F = F + D F (deform.jl:13-16, 35-40), with the unscaled ΔF
        float Fdev[9];     // F - I, exact from the stored state
        if (ACC == 0) {
            double F[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) F[i] = A.P.Fd[i][p];
            float f[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) f[i] = (float)F[i];
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const float inc = D[r] * f[3 * c] + D[r + 3] * f[1 + 3 * c] + D[r + 6] * f[2 + 3 * c];
                    const double nv = F[r + 3 * c] + (double)inc;
                    A.P.Fd[r + 3 * c][p] = nv;
                    Fdev[r + 3 * c] = (float)(nv - (r == c ? 1.0 : 0.0));
                }
        } else {
            float h[9], l[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                h[i] = A.P.Fh[i][p];
                l[i] = A.P.Fl[i][p];
            }
            float inc[9];
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int r = 0; r < 3; ++r) inc[r + 3 * c] = D[r] * h[3 * c] + D[r + 3] * h[1 + 3 * c] + D[r + 6] * h[2 + 3 * c];
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                df_add(h[i], l[i], inc[i]);
                A.P.Fh[i][p] = h[i];
                A.P.Fl[i][p] = l[i];
                const bool dg = i == 0 || i == 4 || i == 8;
                Fdev[i] = dg ? (h[i] - 1.f) + l[i] : h[i] + l[i];
            }
        }
        // Σ N - 1 over the existing nodes (GIMP next to a mesh edge), from the step's half lengths:
        // taken before the domain update rewrites ℓ
        float sm1 = 0.f;
        if (BASIS == EP_BASIS_GIMPM) {
            if (lock) {
                float ms[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) ms[d] = axis_miss<BASIS>(W.a[d], W.o[d], (float)A.g.h[d], A.P.l[d][p]);
                sm1 = -(ms[0] + ms[1] + ms[2]) + (ms[0] * ms[1] + ms[0] * ms[2] + ms[1] * ms[2]) - ms[0] * ms[1] * ms[2];
            }
            gimp_domain<3>(A, p, D, Fdev);
        }
        if (!FIN) {
            // infinitesimal: volume J Ω0 and mass ρ J Ω0 follow J (deform.jl:41-43)
            const float Jm1 = det1p_m1(Fdev);
            const float Om = A.P.Om0[p] + A.P.Om0[p] * Jm1;
            A.P.Om[p] = Om;
            A.P.mp[p] = A.P.rho[p] * Om;
        }
        // F-bar: ΔF <- (ΔJ̄/ΔJ)^(1/3) ΔF (volumetric.jl:23-36), increment form
        if (lock) {
            const float dJp = det1p_m1(D);
            const float r1 = (sm1 + a - dJp) / (1.f + dJp);
            const float s1 = expm1f(log1pf(r1) * (1.f / 3.f));
#pragma unroll
            for (int i = 0; i < 9; ++i) D[i] = D[i] * (1.f + s1) + ((i == 0 || i == 4 || i == 8) ? s1 : 0.f);
        }
        float tt[6];
        bool deferred = false, voigt_done = false;
        if (FIN) {
            R V[3][3], eps[3];
            trial_log_strain3<ACC, R>(A, p, D, V, eps);
            // trial principal Kirchhoff stress τ = Del voigt(ε) (elast.jl:53-54), zero shear
            float tp[6];
#pragma unroll
            for (int i = 0; i < 3; ++i)
                tp[i] = A.Del[i] * (float)eps[0] + A.Del[i + 6] * (float)eps[1] + A.Del[i + 12] * (float)eps[2];
            tp[3] = tp[4] = tp[5] = 0.f;
            bool yielded = false;
            if (plastic_phase) {
                const float ep1f = ACC == 0 ? (float)A.P.ep1d[p] : A.P.ep1h[p] + A.P.ep1l[p];
                const float ep2 = A.cf.nonloc ? A.P.ep2[p] : ep1f;
                if (A.cf.cons == EP_CONS_DP) {
                    if (A.rmode != EP_RMAP_EXACT) {
                        const float coh = fmaxf(A.P.c0[p] + A.Hp * ep2, A.P.cr[p]);
                        const float ef[3] = {(float)eps[0], (float)eps[1], (float)eps[2]};
                        float Vf[3][3];
#pragma unroll
                        for (int i = 0; i < 3; ++i)
#pragma unroll
                            for (int j = 0; j < 3; ++j) Vf[i][j] = (float)V[i][j];
                        const bool ytr = rm_features3(ef, Vf, coh, A.P.tphi[p], A.Gc, A.l2g, fx, fa);
                        deferred = ytr && A.rmode == EP_RMAP_LEARNED;
                    }
                    if (deferred) {
                        emit = true;              // km_rmap_finish3 writes τ, Δλ, ϵpII and b_e
                        ++nplastic;
                    } else {
                        float inc = 0.f;
                        const float dl = dpf6(tp, ep2, A.P.c0[p], A.P.cr[p], A.P.sphi[p], A.P.cphi[p], A.Kc, A.Gc,
                                              A.Hp, &inc);
                        A.P.dlam[p] = dl;
                        yielded = dl != 0.f;
                        if (yielded) add_ep1<ACC>(A, p, inc);
                        if (yielded && A.rmode == EP_RMAP_RECORD) emit = rm_label(fx, (double)A.l2g, fy) != 0;
                    }
                } else {
                    // J2 (J2.jl:21-76) and Cam-Clay: their flow Del n with the tensor shear components of
                    // n is not coaxial with the trial, so they run on the Voigt stress, and b_e is
                    // rebuilt from a second eigen-decomposition of ε = tensor(Del \ τ, ½)
                    {
                        const R td[3] = {(R)tp[0], (R)tp[1], (R)tp[2]};
                        R tv[6];
                        vdv3<R>(V, td, tv);
#pragma unroll
                        for (int i = 0; i < 6; ++i) tt[i] = (float)tv[i];
                    }
                    float newg = 0.f;
                    bool y3 = false;
                    if constexpr (!ITER) y3 = j2f6(tt, ep2, A.P.c0[p], A.P.cr[p], A.Hp, A.Del, &newg) != 0;
                    else newg = cons_iterative<6>(A, p, tt, ep2, &y3);      // modified Cam-Clay (FP64 island)
                    if (y3) {
                        ++nplastic;
                        if (ACC == 0) {
                            A.P.ep1d[p] = (double)newg;
                        } else {
                            A.P.ep1h[p] = newg;
                            A.P.ep1l[p] = 0.f;
                        }
                        float ev[6];
#pragma unroll
                        for (int i = 0; i < 6; ++i) {
                            float acc = 0.f;
#pragma unroll
                            for (int j = 0; j < 6; ++j) acc += A.Cmp[i + 6 * j] * tt[j];
                            ev[i] = acc;
                        }
                        R W[3][3], lam[3];
                        eig_voigt3<R>(ev, W, lam);
                        rebuild_b3<ACC, R>(A, p, W, lam);
                    }
                    voigt_done = true;
                }
                if (yielded) {
                    ++nplastic;
                    // ε = Del \ τ in the principal frame, b = V diag(exp 2ε) V' (DP.jl:63-66)
                    R er[3];
#pragma unroll
                    for (int i = 0; i < 3; ++i)
                        er[i] = (R)(A.Cmp[i] * tp[0] + A.Cmp[i + 6] * tp[1] + A.Cmp[i + 12] * tp[2]);
                    rebuild_b3<ACC, R>(A, p, V, er);
                }
            }
            if (!deferred && !voigt_done) {
                const R td[3] = {(R)tp[0], (R)tp[1], (R)tp[2]};
                R tv[6];
                vdv3<R>(V, td, tv);
#pragma unroll
                for (int i = 0; i < 6; ++i) tt[i] = (float)tv[i];
            }
        } else {
            // σ += Del voigt(sym(ΔF) - I, 2) (+ ωσ - σω for the objective rate)
            float de[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) tt[i] = A.P.tau[i][p];
            de[0] = D[0]; de[1] = D[4]; de[2] = D[8];
            de[3] = D[5] + D[7];        // 2 ε_yz
            de[4] = D[2] + D[6];        // 2 ε_xz
            de[5] = D[1] + D[3];        // 2 ε_xy
            float ds[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                float sacc = 0.f;
#pragma unroll
                for (int j = 0; j < 6; ++j) sacc += A.Del[i + 6 * j] * de[j];
                ds[i] = sacc;
            }
            if (A.cf.jaumann) {
                // W = skew(D); ωσ - σω in Voigt components
                const float w01 = 0.5f * (D[3] - D[1]), w02 = 0.5f * (D[6] - D[2]), w12 = 0.5f * (D[7] - D[5]);
                const float S[3][3] = {{tt[0], tt[5], tt[4]}, {tt[5], tt[1], tt[3]}, {tt[4], tt[3], tt[2]}};
                const float Wm[3][3] = {{0.f, w01, w02}, {-w01, 0.f, w12}, {-w02, -w12, 0.f}};
                float Rm[3][3];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        float sacc = 0.f;
                        for (int q = 0; q < 3; ++q) sacc += Wm[i][q] * S[q][j] - S[i][q] * Wm[q][j];
                        Rm[i][j] = sacc;
                    }
                ds[0] += Rm[0][0]; ds[1] += Rm[1][1]; ds[2] += Rm[2][2];
                ds[3] += Rm[1][2]; ds[4] += Rm[0][2]; ds[5] += Rm[0][1];
            }
#pragma unroll
            for (int i = 0; i < 6; ++i) tt[i] += ds[i];
            if (plastic_phase) {
                const float ep1f = ACC == 0 ? (float)A.P.ep1d[p] : A.P.ep1h[p] + A.P.ep1l[p];
                const float ep2 = A.cf.nonloc ? A.P.ep2[p] : ep1f;
                if (A.cf.cons == EP_CONS_DP) {
                    float inc = 0.f;
                    const float dl = dpf6(tt, ep2, A.P.c0[p], A.P.cr[p], A.P.sphi[p], A.P.cphi[p], A.Kc, A.Gc, A.Hp, &inc);
                    A.P.dlam[p] = dl;
                    if (dl != 0.f) {
                        ++nplastic;
                        add_ep1<ACC>(A, p, inc);
                    }
                } else {
                    float newg = 0.f;
                    bool y3 = false;
                    if constexpr (!ITER) y3 = j2f6(tt, ep2, A.P.c0[p], A.P.cr[p], A.Hp, A.Del, &newg) != 0;
                    else newg = cons_iterative<6>(A, p, tt, ep2, &y3);      // modified Cam-Clay (FP64 island)
                    if (y3) {
                        ++nplastic;
                        if (ACC == 0) {
                            A.P.ep1d[p] = (double)newg;
                        } else {
                            A.P.ep1h[p] = newg;
                            A.P.ep1l[p] = 0.f;
                        }
                    }
                }
            }
        }
        if (!deferred) {
            bool okv = true;
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                A.P.tau[i][p] = tt[i];
                okv = okv && isfinite(tt[i]);
            }
            if (!okv) set_err(A.ctl, EP_ERR_NONFINITE, p);
        }
        if (!lock) place_next(A, p, nxt);
        if (bad) set_err(A.ctl, EP_ERR_INVALID_POSITION, W.c);
    }
    // learned map slots / recorded pairs: one atomic per warp for the warp's points
    if (FIN && A.rmode != EP_RMAP_EXACT) {
        const unsigned bal = __ballot_sync(0xffffffffu, emit);
        if (bal) {
            const int lane = threadIdx.x & 31;
            const unsigned below = bal & ((1u << lane) - 1u);
            if (A.rmode == EP_RMAP_LEARNED) {
                int base = 0;
                if (lane == 0) base = atomicAdd(A.rcount, __popc(bal));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (emit) {
                    const int slot = base + __popc(below);
                    float4* dx = reinterpret_cast<float4*>(A.rx + (size_t)slot * RM_NX);
                    dx[0] = make_float4(fx[0], fx[1], fx[2], fx[3]);
                    dx[1] = make_float4(fx[4], fx[5], fx[6], fx[7]);
                    float4* da = reinterpret_cast<float4*>(A.raux + (size_t)slot * 12);
                    da[0] = make_float4(fa[0], fa[1], fa[2], fa[3]);
                    da[1] = make_float4(fa[4], fa[5], fa[6], fa[7]);
                    da[2] = make_float4(fa[8], fa[9], fa[10], fa[11]);
                    A.rpt[slot] = fp;
                }
            } else {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd((unsigned long long*)A.rec_count, (unsigned long long)__popc(bal));
                base = __shfl_sync(0xffffffffu, base, 0);
                const long long slot = (long long)base + __popc(below);
                if (emit && slot < A.rec_cap) {
                    float4* dx = reinterpret_cast<float4*>(A.rx + (size_t)slot * RM_NX);
                    dx[0] = make_float4(fx[0], fx[1], fx[2], fx[3]);
                    dx[1] = make_float4(fx[4], fx[5], fx[6], fx[7]);
                    *reinterpret_cast<float4*>(A.ry + (size_t)slot * RM_NY) = make_float4(fy[0], fy[1], fy[2], fy[3]);
                }
            }
        }
    }
    const int tot = __reduce_add_sync(0xffffffffu, nplastic);
    if ((threadIdx.x & 31) == 0 && tot) atomicAdd((unsigned long long*)&A.ctl->plastic, (unsigned long long)tot);
}

// rmap_fallback_slot3_32: the rejected 3d slots' return as the exact-map 3d step runs it (dpf6, the
// outer-cone Drucker-Prager return of DP.jl:69-98 in FP32, on the principal trial rebuilt from the
// slot), then b_e and τ rebuilt in the trial's frame as km_rmap_finish3 does for accepted slots
template <int ACC>
__device__ __noinline__ void rmap_fallback_slot3_32(const MCtx& A, int i) {
    using R = typename std::conditional<ACC == 0, double, float>::type;
    const float4 x0 = *reinterpret_cast<const float4*>(A.rx + (size_t)i * RM_NX);
    const float* ax = A.raux + (size_t)i * 12;
    const int p = A.rpt[i];
    const float s = ax[9], coh = ax[10];
    const float te[3] = {s * x0.x, s * x0.y, s * x0.z};
    float tt[6];
    for (int a = 0; a < 3; ++a) tt[a] = A.Del[a] * te[0] + A.Del[a + 6] * te[1] + A.Del[a + 12] * te[2];
    tt[3] = tt[4] = tt[5] = 0.f;
    float inc = 0.f;
    const float dl = dpf6(tt, 0.f, coh, 0.f, A.P.sphi[p], A.P.cphi[p], A.Kc, A.Gc, 0.f, &inc);
    A.P.dlam[p] = dl;
    add_ep1<ACC>(A, p, inc);
    R V[3][3], td[3], tv[6];
    for (int c = 0; c < 3; ++c) {
        td[c] = (R)tt[c];
        for (int r = 0; r < 3; ++r) V[r][c] = (R)ax[r + 3 * c];
    }
    if (dl != 0.f) {
        R er[3];
        for (int a = 0; a < 3; ++a) er[a] = (R)(A.Cmp[a] * tt[0] + A.Cmp[a + 6] * tt[1] + A.Cmp[a + 12] * tt[2]);
        rebuild_b3<ACC, R>(A, p, V, er);
    }
    vdv3<R>(V, td, tv);
    bool okv = true;
    for (int q = 0; q < 6; ++q) {
        A.P.tau[q][p] = (float)tv[q];
        okv = okv && isfinite(tv[q]);
    }
    if (!okv) set_err(A.ctl, EP_ERR_NONFINITE, p);
}

// km_rmap_finish3: the network's returned principal strains for the slots of km_cons3 (3d),
// accepted under the tests of km_rmap_finish (compressive side of the apex, on the yield
// surface and at the trial mean stress within 1e-3 c, principal order kept, Δλ >= 0)
template <int ACC>
__global__ void __launch_bounds__(256) km_rmap_finish3(MCtx A) {
    using R = typename std::conditional<ACC == 0, double, float>::type;
    EP_ACTIVE(A.ctl);
    const int n = *A.rcount;
    int nl = 0, nf = 0;
    for (int i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
    const int i = i0 + threadIdx.x;
    bool reject = false;
    if (i < n) {
        const float4 x0 = *reinterpret_cast<const float4*>(A.rx + (size_t)i * RM_NX);
        const float4 x1 = *reinterpret_cast<const float4*>(A.rx + (size_t)i * RM_NX + 4);
        const float4 y = *reinterpret_cast<const float4*>(A.ry + (size_t)i * RM_NY);
        const float* ax = A.raux + (size_t)i * 12;
        const float s = ax[9], coh = ax[10];
        const float tphi = x1.x, phin = x1.z;
        const float rr = rsqrtf(1.f + tphi * tphi), sphi = tphi * rr, cphi = rr;
        const float eta = 6.f * sphi / (1.7320508075688772f * (3.f + sphi));
        const float xi = 6.f * coh * cphi / (1.7320508075688772f * (3.f + sphi));
        bool ok = phin >= (float)RM_PHI_MIN && isfinite(y.x) && isfinite(y.y) && isfinite(y.z);
        float e[3] = {0.f, 0.f, 0.f}, tp[3] = {0.f, 0.f, 0.f}, dl = 0.f;
        if (ok) {
            const float xs[3] = {x0.x, x0.y, x0.z};
            // the correction in the trial's frame (ep_rmap.h rm_frame3); tan ψ = 0: the exact
            // return shrinks the deviator radially (DP.jl:81-86), so only the component along the
            // trial deviator q is kept (in 2d this is the deviatoric projection of km_rmap_finish)
            float fm[3], fq[3], fr[3];
            rm_frame3<float>(xs[0], xs[1], xs[2], fm, fq, fr);
            const float c0 = x1.y == 0.f ? 0.f : y.x, c2 = x1.y == 0.f ? 0.f : y.z;
            float yv[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) yv[j] = c0 * fm[j] + y.y * fq[j] + c2 * fr[j];
#pragma unroll
            for (int j = 0; j < 3; ++j) e[j] = s * (xs[j] + phin * yv[j]);
#pragma unroll
            for (int j = 0; j < 3; ++j) tp[j] = A.Del[j] * e[0] + A.Del[j + 6] * e[1] + A.Del[j + 12] * e[2];
            const float P = (tp[0] + tp[1] + tp[2]) * (1.f / 3.f);
            const float d0 = tp[0] - P, d1 = tp[1] - P, d2 = tp[2] - P;
            const float tII = sqrtf(0.5f * (d0 * d0 + d1 * d1 + d2 * d2));
            const float fs = tII + eta * P - xi;
            const float xm = (xs[0] + xs[1] + xs[2]) * (1.f / 3.f);
            const float q0 = xs[0] - xm, q1 = xs[1] - xm, q2 = xs[2] - xm;
            const float tIItr = coh * sqrtf(0.5f * (q0 * q0 + q1 * q1 + q2 * q2));
            dl = (tIItr - tII) / A.Gc;                          // ψ = 0: Δλ = (τII,trial - τII) / G
            const float Ptr = coh * (A.l2g + (1.f / 3.f)) * (xs[0] + xs[1] + xs[2]);
            const bool below_apex = tphi > 0.f ? Ptr < coh / tphi : true;
            ok = fabsf(fs) <= 1.0e-3f * coh && fabsf(P - Ptr) <= 1.0e-3f * coh && dl >= 0.f && e[0] >= e[1] &&
                 e[1] >= e[2] && below_apex && isfinite(fs);
        }
        if (ok) {
            ++nl;
            const int p = A.rpt[i];
            add_ep1<ACC>(A, p, dl * 0.57735026918962576f);
            A.P.dlam[p] = dl;
            R V[3][3], er[3], td[3], tv[6];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                er[c] = (R)e[c];
                td[c] = (R)tp[c];
#pragma unroll
                for (int r = 0; r < 3; ++r) V[r][c] = (R)ax[r + 3 * c];
            }
            rebuild_b3<ACC, R>(A, p, V, er);
            vdv3<R>(V, td, tv);
#pragma unroll
            for (int k = 0; k < 6; ++k) A.P.tau[k][p] = (float)tv[k];
        } else {
            reject = true;
        }
    }
    // rejected slots: the exact return right here (a few per thousand slots, in FP32 as the exact-map
    // step runs it)
    if (reject) {
        rmap_fallback_slot3_32<ACC>(A, i);
        ++nf;
    }
    }
    const int tl = __reduce_add_sync(0xffffffffu, nl), tf = __reduce_add_sync(0xffffffffu, nf);
    if ((threadIdx.x & 31) == 0 && tl) atomicAdd(&A.ctl->rm_learned, (unsigned long long)tl);
    if ((threadIdx.x & 31) == 0 && tf) atomicAdd(&A.ctl->rm_fallback, (unsigned long long)tf);
}

// ===========================================================================
// Batched ensemble as one persistent kernel (config 4): n independent 2d mixed-step instances, each
// with its own mesh, points, control block and time window, advanced by one cooperative kernel that
// loops over up to `steps` steps; each phase of the step (the kernels of mixed_step_impl) walks the
// virtual blocks of all instances (instance i owns blocks off[i] .. off[i+1] - 1), and a grid barrier
// separates the phases.  Instances past their window return from every phase at once (EP_ACTIVE).
// Barrier waits are bounded (1 s, %globaltimer); a wait that gives up sets the error word, and every
// block then skips the remaining phases.
struct BInst {
    float* gz;              // m, p, f of the instance's nodes (zeroed at each step start)
    long long gzn;
    int* sz;                // both parities' cell counts and the cursor
    long long szn;
};

struct BatchArgs {
    const MCtx* ctx;        // n argument blocks
    const BInst* inst;
    int n;
    const int* off;         // 3 (n + 1): virtual-block prefix sums of P2G tiles, point blocks, node blocks
    int steps;
    int plastic_phase;
    int any_musl, any_lock;
    int keep_ctl;           // 1: dt and g as the host set them (the autotuner's dt = 0 steps)
    unsigned* bar;          // [0] arrivals, [1] generation
    int* err;
};

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// grid-wide barrier of the cooperative launch (all blocks resident): arrival counter and generation
__device__ __forceinline__ bool grid_sync(const BatchArgs& B) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = *(volatile int*)B.err == 0;
        if (ok) {
            volatile unsigned* gen = B.bar + 1;
            const unsigned g = *gen;
            __threadfence();
            const unsigned arrived = atomicAdd(B.bar, 1u) + 1u;
            if (arrived == gridDim.x) {
                atomicExch(B.bar, 0u);
                __threadfence();
                atomicAdd(B.bar + 1, 1u);
            } else {
                const unsigned long long t0 = gtimer();
                while (*gen == g) {
                    if (*(volatile int*)B.err) {
                        ok = 0;
                        break;
                    }
                    if (gtimer() - t0 > 1000000000ull) {
                        atomicExch(B.err, 1);
                        ok = 0;
                        break;
                    }
                    __nanosleep(100);
                }
            }
            __threadfence();
        }
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

// the instance owning virtual block vb: the largest i with off[i] <= vb (off[n] > vb)
__device__ __forceinline__ int inst_of(const int* off, int n, int vb) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= vb) lo = mid;
        else hi = mid;
    }
    return lo;
}

// the next-step cell starts of one instance by one block (count[nxt] -> start[nxt], total at ncell)
__device__ __forceinline__ void scan_block_body(const MCtx& A) {
    EP_ACTIVE(A.ctl);
    const int par = A.ctl->parity ^ 1;
    const int n = A.g.ncell;
    const int* in = A.S.count[par];
    int* out = A.S.start[par];
    int run = 0;
    for (int c0 = 0; c0 < n; c0 += blockDim.x * MSCAN_IPT) {
        const int base = c0 + threadIdx.x * MSCAN_IPT;
        int v[MSCAN_IPT], sum = 0;
#pragma unroll
        for (int i = 0; i < MSCAN_IPT; ++i) {
            v[i] = base + i < n ? in[base + i] : 0;
            sum += v[i];
        }
        int tot;
        int ex = mblock_scan(sum, &tot) + run;
#pragma unroll
        for (int i = 0; i < MSCAN_IPT; ++i) {
            if (base + i < n) out[base + i] = ex;
            ex += v[i];
        }
        run += tot;
    }
    if (threadIdx.x == 0) out[n] = run;
}

template <int BASIS, int ACC, int TC>
__global__ void __launch_bounds__(256, 3) km_batch_steps(BatchArgs B) {
    const int n = B.n;
    const int* offT = B.off;
    const int* offP = B.off + (n + 1);
    const int* offN = B.off + 2 * (n + 1);
    const int nT = offT[n], nP = offP[n], nN = offN[n];
    bool ok = true;
    for (int st = 0; st < B.steps && ok; ++st) {
        // step start: control blocks (ctl_begin_run) and the zeroed accumulators of mixed_step_impl
        for (int i = blockIdx.x; i < n; i += gridDim.x) {
            const MCtx& A = B.ctx[i];
            if (threadIdx.x == 0 && !B.keep_ctl) ctl_begin_run(A.ctl, A.g.dim, A.g.h[0], A.g.h[1], A.g.h[2], A.c);
            const BInst& I = B.inst[i];
            for (long long k = threadIdx.x; k < I.gzn; k += blockDim.x) I.gz[k] = 0.f;
            for (long long k = threadIdx.x; k < I.szn; k += blockDim.x) I.sz[k] = 0;
        }
        if (!(ok = grid_sync(B))) break;
        for (int vb = blockIdx.x; vb < nT; vb += gridDim.x) {
            const int i = inst_of(offT, n, vb);
            p2g_tile_body<BASIS, TC, false, 256>(B.ctx[i], vb - offT[i]);
        }
        if (!(ok = grid_sync(B))) break;
        for (int vb = blockIdx.x; vb < nN; vb += gridDim.x) {
            const int i = inst_of(offN, n, vb);
            solve_body(B.ctx[i], vb - offN[i]);
        }
        if (!(ok = grid_sync(B))) break;
        for (int vb = blockIdx.x; vb < nP; vb += gridDim.x) {
            const int i = inst_of(offP, n, vb);
            g2p_seg_body<BASIS, false>(B.ctx[i], vb - offP[i]);
        }
        if (!(ok = grid_sync(B))) break;
        if (B.any_musl) {
            for (int vb = blockIdx.x; vb < nN; vb += gridDim.x) {
                const int i = inst_of(offN, n, vb);
                if (B.ctx[i].cf.musl) vmusl_body(B.ctx[i], vb - offN[i]);
            }
            if (!(ok = grid_sync(B))) break;
        }
        for (int i = blockIdx.x; i < n; i += gridDim.x) scan_block_body(B.ctx[i]);
        if (!(ok = grid_sync(B))) break;
        if (B.any_lock) {
            for (int vb = blockIdx.x; vb < nP; vb += gridDim.x) {
                const int i = inst_of(offP, n, vb);
                if (B.ctx[i].cf.locking) fbar_seg_body<BASIS, false>(B.ctx[i], vb - offP[i]);
            }
            if (!(ok = grid_sync(B))) break;
            for (int vb = blockIdx.x; vb < nN; vb += gridDim.x) {
                const int i = inst_of(offN, n, vb);
                if (B.ctx[i].cf.locking) dJn_body(B.ctx[i], vb - offN[i]);
            }
            if (!(ok = grid_sync(B))) break;
        }
        for (int vb = blockIdx.x; vb < nP; vb += gridDim.x) {
            const int i = inst_of(offP, n, vb);
            if (B.ctx[i].P.np > 0) cons_body<BASIS, ACC>(B.ctx[i], vb - offP[i], B.plastic_phase);
        }
        if (!(ok = grid_sync(B))) break;
        // step end: parity flip (km_flip) and t += dt (ctl_end)
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            Ctl* c = B.ctx[i].ctl;
            if (c->active) c->parity ^= 1;
            ctl_end(c);
        }
        if (!(ok = grid_sync(B))) break;
    }
}

// The same phases as kernels of their own over all instances (one launch per phase and step,
// 16 steps per graph): no grid barriers, each phase at its own occupancy.
__global__ void __launch_bounds__(256) kb_begin(BatchArgs B) {
    const int i = blockIdx.x;
    const MCtx& A = B.ctx[i];
    if (threadIdx.x == 0 && !B.keep_ctl) ctl_begin_run(A.ctl, A.g.dim, A.g.h[0], A.g.h[1], A.g.h[2], A.c);
    const BInst& I = B.inst[i];
    for (long long k = threadIdx.x; k < I.gzn; k += blockDim.x) I.gz[k] = 0.f;
    for (long long k = threadIdx.x; k < I.szn; k += blockDim.x) I.sz[k] = 0;
}
template <int BASIS, int TC>
__global__ void __launch_bounds__(4 * TC) kb_p2g(BatchArgs B) {
    const int vb = blockIdx.x, i = inst_of(B.off, B.n, vb);
    p2g_tile_body<BASIS, TC, false>(B.ctx[i], vb - B.off[i]);
}
__global__ void __launch_bounds__(256) kb_solve(BatchArgs B) {
    const int* o = B.off + 2 * (B.n + 1);
    const int vb = blockIdx.x, i = inst_of(o, B.n, vb);
    solve_body(B.ctx[i], vb - o[i]);
}
template <int BASIS>
__global__ void __launch_bounds__(256) kb_g2p(BatchArgs B) {
    const int* o = B.off + (B.n + 1);
    const int vb = blockIdx.x, i = inst_of(o, B.n, vb);
    g2p_seg_body<BASIS, false>(B.ctx[i], vb - o[i]);
}
__global__ void __launch_bounds__(256) kb_vmusl(BatchArgs B) {
    const int* o = B.off + 2 * (B.n + 1);
    const int vb = blockIdx.x, i = inst_of(o, B.n, vb);
    if (B.ctx[i].cf.musl) vmusl_body(B.ctx[i], vb - o[i]);
}
__global__ void __launch_bounds__(256) kb_scan(BatchArgs B) { scan_block_body(B.ctx[blockIdx.x]); }
template <int BASIS>
__global__ void __launch_bounds__(256) kb_fbar(BatchArgs B) {
    const int* o = B.off + (B.n + 1);
    const int vb = blockIdx.x, i = inst_of(o, B.n, vb);
    if (B.ctx[i].cf.locking) fbar_seg_body<BASIS, false>(B.ctx[i], vb - o[i]);
}
__global__ void __launch_bounds__(256) kb_dJn(BatchArgs B) {
    const int* o = B.off + 2 * (B.n + 1);
    const int vb = blockIdx.x, i = inst_of(o, B.n, vb);
    if (B.ctx[i].cf.locking) dJn_body(B.ctx[i], vb - o[i]);
}
template <int BASIS, int ACC>
__global__ void __launch_bounds__(256) kb_cons(BatchArgs B) {
    const int* o = B.off + (B.n + 1);
    const int vb = blockIdx.x, i = inst_of(o, B.n, vb);
    if (B.ctx[i].P.np > 0) cons_body<BASIS, ACC>(B.ctx[i], vb - o[i], B.plastic_phase);
}
__global__ void kb_end(BatchArgs B) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < B.n) {
        Ctl* c = B.ctx[i].ctl;
        if (c->active) c->parity ^= 1;
        ctl_end(c);
    }
}

template <int BASIS, int ACC, int TC>
static void batch_phase_steps_t(const BatchArgs& a, const int* nblk, int steps, cudaStream_t s) {
    const int n = a.n;
    for (int st = 0; st < steps; ++st) {
        kb_begin<<<n, 256, 0, s>>>(a);
        kb_p2g<BASIS, TC><<<nblk[0], 4 * TC, 0, s>>>(a);
        kb_solve<<<nblk[2], 256, 0, s>>>(a);
        kb_g2p<BASIS><<<nblk[1], 256, 0, s>>>(a);
        if (a.any_musl) kb_vmusl<<<nblk[2], 256, 0, s>>>(a);
        kb_scan<<<n, 256, 0, s>>>(a);
        if (a.any_lock) {
            kb_fbar<BASIS><<<nblk[1], 256, 0, s>>>(a);
            kb_dJn<<<nblk[2], 256, 0, s>>>(a);
        }
        kb_cons<BASIS, ACC><<<nblk[1], 256, 0, s>>>(a);
        kb_end<<<(n + 255) / 256, 256, 0, s>>>(a);
    }
}

struct BatchImpl {
    MCtx* ctx = nullptr;
    BInst* inst = nullptr;
    int* off = nullptr;
    unsigned* bar = nullptr;
    int* err = nullptr;
    int n = 0, basis = 0, acc = 0, any_musl = 0, any_lock = 0;
    int grid[3] = {0, 0, 0};      // resident blocks per tile shape 16 / 32 / 64
    int nblk[3][3] = {};          // per tile shape: total virtual blocks of tiles, points, nodes
};

template <int BASIS, int ACC, int TC>
static const void* batch_fn() {
    return (const void*)km_batch_steps<BASIS, ACC, TC>;
}

template <int BASIS, int ACC>
static const void* batch_fn_tc(int tile) {
    return tile == 16 ? batch_fn<BASIS, ACC, 16>() : (tile == 32 ? batch_fn<BASIS, ACC, 32>() : batch_fn<BASIS, ACC, 64>());
}

static const void* batch_kernel(int basis, int acc, int tile) {
    if (basis == EP_BASIS_BSMPM) return acc ? batch_fn_tc<EP_BASIS_BSMPM, 1>(tile) : batch_fn_tc<EP_BASIS_BSMPM, 0>(tile);
    if (basis == EP_BASIS_GIMPM) return acc ? batch_fn_tc<EP_BASIS_GIMPM, 1>(tile) : batch_fn_tc<EP_BASIS_GIMPM, 0>(tile);
    return acc ? batch_fn_tc<EP_BASIS_SMPM, 1>(tile) : batch_fn_tc<EP_BASIS_SMPM, 0>(tile);
}

__global__ void km_batch_flags(const MCtx* ctx, int n, const int* berr, int* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const Ctl* c = ctx[i].ctl;
        flags[i] = (c->active ? 1 : 0) | (c->err ? 2 : 0) | (*berr ? 4 : 0);
    }
}

// one 3d step; DET = no floating-point atomics (per-cell partials + node gathers, point-id ordered lists)
template <int BASIS, int ACC, bool DET>
static void mixed_step3_impl(const MixedCtx& X, int phase, cudaStream_t s) {
    const MCtx& A = *(const MCtx*)X.impl;
    const int nc = A.g.ncell, nn = A.g.nnode, np = A.P.np;
    const int gn = (nn + 255) / 256, gp = (np + 255) / 256, gc = (nc + 255) / 256, gt = (nc + 15) / 16;
    const int gs = gp > 0 ? gp : 1;
    Prof* pr = (X.prof && X.prof->on) ? X.prof : nullptr;
    auto mark = [&](const char* nm) {
        if (pr) pr->mark(nm, s);
    };
    long long L = 0;
    launch_zero(X, s);
    ++L;
    mark("memset");
    km_p2g_tile3<BASIS, 16, DET><<<gt, 256, 0, s>>>(A);
    if (DET) {
        km_gather3<7><<<gn, 256, 0, s>>>(A, A.N.m, A.N.p[0], A.N.p[1], A.N.p[2], A.N.f[0], A.N.f[1], A.N.f[2]);
        ++L;
    }
    mark("p2g");
    km_solve<<<gn, 256, 0, s>>>(A);
    mark("solve");
    if (A.cf.trsfr == EP_TRSFR_APIC) km_g2p_seg3<BASIS, DET, true><<<gs, 256, 0, s>>>(A);
    else km_g2p_seg3<BASIS, DET, false><<<gs, 256, 0, s>>>(A);
    mark("g2p");
    if (X.ev_moved) hook_record(X.ev_moved, s, X.hooks_internal);
    L += 3;
    if (A.cf.musl) {
        if (DET) {
            km_aux_tile3<BASIS, 16, 1><<<gt, 256, 0, s>>>(A);
            km_gather3<3><<<gn, 256, 0, s>>>(A, A.N.pm[0], A.N.pm[1], A.N.pm[2], nullptr, nullptr, nullptr, nullptr);
            mark("musl");
            L += 2;
        }
    }
    launch_vmusl_scan(A, A.cf.musl, s);
    mark("vmusl_scan");
    ++L;
    if (A.cf.locking) {
        km_fbar_seg3<BASIS, DET><<<gs, 256, 0, s>>>(A);
        if (DET) {
            km_aux_tile3<BASIS, 16, 2><<<gt, 256, 0, s>>>(A);
            km_gather3<1><<<gn, 256, 0, s>>>(A, A.N.dJacc, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
            L += 2;
        }
        mark("fbar");
        km_dJn<<<gn, 256, 0, s>>>(A);
        mark("dJn");
        L += 2;
    }
    if (X.ev_need) hook_wait(s, X.ev_need, X.hooks_internal);   // the constitutive pass's other inputs
    if (np > 0 && A.cf.nonloc && phase == EP_PHASE_ELASTOPLASTIC) {
        km_nonlocal3<ACC><<<np, 32, 0, s>>>(A);
        mark("nonlocal");
        ++L;
    }
    if (np > 0) {
        const int pp = phase == EP_PHASE_ELASTOPLASTIC;
        const bool iter = A.cf.cons == EP_CONS_CAMC;
        if (A.cf.deform == EP_DEFORM_FINITE) {
            if (iter) km_cons3<BASIS, ACC, true, true><<<gp, 256, 0, s>>>(A, pp);
            else km_cons3<BASIS, ACC, true><<<gp, 256, 0, s>>>(A, pp);
        } else if (iter) {
            km_cons3<BASIS, ACC, false, true><<<gp, 256, 0, s>>>(A, pp);
        } else {
            km_cons3<BASIS, ACC, false><<<gp, 256, 0, s>>>(A, pp);
        }
        mark("cons");
        ++L;
        if (A.rmode == EP_RMAP_LEARNED && X.net && phase == EP_PHASE_ELASTOPLASTIC) {
            mlp_infer(X.net, A.rx, A.rcount, np, A.ry, s);
            mark("mlp");
            km_rmap_finish3<ACC><<<std::min(gp, 4 * sm_count()), 256, 0, s>>>(A);
            mark("rmap_finish");
            L += 2;
        }
    }
    if (DET) {
        km_sort_cells<<<gc, 256, 0, s>>>(A, 0);   // the next step's lists in point-id order
        mark("sort");
        ++L;
    }
    const bool lrn = A.rmode == EP_RMAP_LEARNED;
    km_flip<<<1, 1, 0, s>>>(A.ctl, lrn ? A.rcount : nullptr, lrn ? A.fbcount : nullptr);
    ++L;
    if (X.launches) *X.launches += L;
}

// ---------------------------------------------------------------------------
template <int BASIS, int TC, int KIND>
static void launch_tile(const MCtx& A, cudaStream_t s) {
    const int nc = A.g.ncell;
    if (KIND == 0) km_p2g_tile<BASIS, TC, true><<<(nc + TC - 1) / TC, 4 * TC, 0, s>>>(A);
    else km_aux_tile<BASIS, TC, KIND><<<(nc + TC - 1) / TC, 4 * TC, 0, s>>>(A);
}

// one step of the mixed path; DET = no floating-point atomics (per-cell partials + node gathers)
template <int BASIS, int ACC, bool DET>
static void mixed_step_impl(const MixedCtx& X, int phase, cudaStream_t s) {
    const MCtx& A = *(const MCtx*)X.impl;
    const int nc = A.g.ncell, nn = A.g.nnode, np = A.P.np;
    const int gn = (nn + 255) / 256, gp = (np + 255) / 256, gc = (nc + 255) / 256;
    const int gs = gp > 0 ? gp : 1;   // point-parallel transfers (an empty list still launches)
    Prof* pr = (X.prof && X.prof->on) ? X.prof : nullptr;
    auto mark = [&](const char* nm) {
        if (pr) pr->mark(nm, s);
    };
    auto tile = [&](auto kind) {
        constexpr int K = decltype(kind)::value;
        if (X.p2g_tile == 16) launch_tile<BASIS, 16, K>(A, s);
        else if (X.p2g_tile == 32) launch_tile<BASIS, 32, K>(A, s);
        else launch_tile<BASIS, 64, K>(A, s);
    };
    long long L = 0;
    launch_zero(X, s);                // node accumulators, both parities' counts, cursor, scan words
    mark("zero");
    ++L;
    if (DET) {
        tile(std::integral_constant<int, 0>());
        km_gather<5><<<gn, 256, 0, s>>>(A, A.N.m, A.N.p[0], A.N.p[1], A.N.f[0], A.N.f[1]);
        L += 1;
    } else if (X.p2g_tile == 16) launch_pdl(km_p2g_tile<BASIS, 16, false>, (nc + 15) / 16, 64, s, A);
    else if (X.p2g_tile == 32) launch_pdl(km_p2g_tile<BASIS, 32, false>, (nc + 31) / 32, 128, s, A);
    else launch_pdl(km_p2g_tile<BASIS, 64, false>, (nc + 63) / 64, 256, s, A);
    mark("p2g");
    // G2P with the mUSL momentum scatter fused in (tile form), or G2P then a separate mUSL scatter;
    // the tile form with the grid update on chip when every tile's node box fits
    const bool g2p_musl = !DET && A.cf.musl && A.cf.trsfr != EP_TRSFR_APIC;
    const bool solve_fused = g2p_musl && max_tile_box(A.g, X.p2g_tile) <= TB_SOLVE;
    if (!solve_fused) {
        launch_pdl(km_solve, gn, 256, s, A);
        mark("solve");
        ++L;
    }
    if (solve_fused) {
        if (X.p2g_tile == 16) launch_pdl(km_g2p_tile<BASIS, 16, true>, (nc + 15) / 16, 64, s, A);
        else if (X.p2g_tile == 32) launch_pdl(km_g2p_tile<BASIS, 32, true>, (nc + 31) / 32, 128, s, A);
        else launch_pdl(km_g2p_tile<BASIS, 64, true>, (nc + 63) / 64, 256, s, A);
    } else if (g2p_musl) {
        if (X.p2g_tile == 16) launch_pdl(km_g2p_tile<BASIS, 16>, (nc + 15) / 16, 64, s, A);
        else if (X.p2g_tile == 32) launch_pdl(km_g2p_tile<BASIS, 32>, (nc + 31) / 32, 128, s, A);
        else launch_pdl(km_g2p_tile<BASIS, 64>, (nc + 63) / 64, 256, s, A);
    } else if (DET) {
        km_g2p_seg<BASIS, true><<<gs, 256, 0, s>>>(A);
    } else {
        km_g2p_seg<BASIS, false, false><<<gs, 256, 0, s>>>(A);
    }
    mark("g2p");
    L += 2;                           // P2G, G2P
    if (X.ev_moved) hook_record(X.ev_moved, s, X.hooks_internal);   // positions and velocities final
    if (A.cf.musl && !g2p_musl) {
        if (DET) {
            tile(std::integral_constant<int, 1>());
            km_gather<2><<<gn, 256, 0, s>>>(A, A.N.pm[0], A.N.pm[1], nullptr, nullptr, nullptr);
            mark("musl");
            L += 2;
        } else {
            // the mUSL momentum P2G (augm.jl:13-25) in the tile form, FP32 atomics per node
            if (X.p2g_tile == 16) km_aux_tile<BASIS, 16, 1, true><<<(nc + 15) / 16, 64, 0, s>>>(A);
            else if (X.p2g_tile == 32) km_aux_tile<BASIS, 32, 1, true><<<(nc + 31) / 32, 128, 0, s>>>(A);
            else km_aux_tile<BASIS, 64, 1, true><<<(nc + 63) / 64, 256, 0, s>>>(A);
            mark("musl");
            ++L;
        }
    }
    // the mUSL nodal velocity and the next step's cell offsets in one launch (the velocity formed by
    // the F-bar kernel instead when the grid update ran in the G2P)
    const bool vm_fused = solve_fused && A.cf.locking;
    launch_vmusl_scan(A, A.cf.musl && !vm_fused, s);
    mark("vmusl_scan");
    ++L;
    if (A.cf.locking) {
        if (DET) km_fbar_seg<BASIS, true><<<gs, 256, 0, s>>>(A);
        else if (vm_fused) {
            if (X.p2g_tile == 16) launch_pdl(km_fbar_tile<BASIS, 16, true>, (nc + 15) / 16, 64, s, A);
            else if (X.p2g_tile == 32) launch_pdl(km_fbar_tile<BASIS, 32, true>, (nc + 31) / 32, 128, s, A);
            else launch_pdl(km_fbar_tile<BASIS, 64, true>, (nc + 63) / 64, 256, s, A);
        } else if (X.p2g_tile == 16) launch_pdl(km_fbar_tile<BASIS, 16>, (nc + 15) / 16, 64, s, A);
        else if (X.p2g_tile == 32) launch_pdl(km_fbar_tile<BASIS, 32>, (nc + 31) / 32, 128, s, A);
        else launch_pdl(km_fbar_tile<BASIS, 64>, (nc + 63) / 64, 256, s, A);
        ++L;
        mark("fbar");
        if (DET) {
            // the deterministic partials, their fixed-order node sums and the nodal δJ
            tile(std::integral_constant<int, 2>());
            km_gather<1><<<gn, 256, 0, s>>>(A, A.N.dJacc, nullptr, nullptr, nullptr, nullptr);
            km_dJn<<<gn, 256, 0, s>>>(A);
            mark("dJn");
            L += 3;
        }
    }
    if (X.ev_need) hook_wait(s, X.ev_need, X.hooks_internal);   // the constitutive pass's other inputs
    if (np > 0 && A.cf.nonloc && phase == EP_PHASE_ELASTOPLASTIC) {
        km_nonlocal<ACC><<<np, 32, 0, s>>>(A);
        mark("nonlocal");
        ++L;
    }
    const bool net = A.rmode == EP_RMAP_LEARNED && X.net && phase == EP_PHASE_ELASTOPLASTIC;
    // the parity flip rides on the constitutive kernel's last block unless later kernels of the step
    // (the network, the deterministic list sort) still read the current parity
    const bool flip_in_cons = np > 0 && !DET && !net;
    const bool flip_in_finish = np > 0 && !DET && net;     // the learned map's finish kernel is last
    if (np > 0) {
        const int pp = phase == EP_PHASE_ELASTOPLASTIC;
        const bool iter = A.cf.cons == EP_CONS_MC || A.cf.cons == EP_CONS_CAMC;
        if (iter && flip_in_cons) launch_pdl(km_cons<BASIS, ACC, true, true>, gp, 256, s, A, pp);
        else if (iter) launch_pdl(km_cons<BASIS, ACC, false, true>, gp, 256, s, A, pp);
        else if (flip_in_cons) launch_pdl(km_cons<BASIS, ACC, true>, gp, 256, s, A, pp);
        else launch_pdl(km_cons<BASIS, ACC>, gp, 256, s, A, pp);
        mark("cons");
        ++L;
        if (net) {
            mlp_infer(X.net, A.rx, A.rcount, np, A.ry, s);
            mark("mlp");
            const int gf = std::min(gp, 4 * sm_count());
            // plain launches: as programmatic dependents the network and finish kernels made the
            // learned step slower (0.162 against 0.157 ms per c2 step)
            if (flip_in_finish) km_rmap_finish<ACC, true><<<gf, 256, 0, s>>>(A);
            else km_rmap_finish<ACC><<<gf, 256, 0, s>>>(A);
            mark("rmap_finish");
            L += 2;
        }
    }
    if (DET) {
        km_sort_cells<<<gc, 256, 0, s>>>(A, 0);   // the next step's lists in point-id order
        mark("sort");
        ++L;
    }
    if (!flip_in_cons && !flip_in_finish) {
        const bool lrn = A.rmode == EP_RMAP_LEARNED;
        km_flip<<<1, 1, 0, s>>>(A.ctl, lrn ? A.rcount : nullptr, lrn ? A.fbcount : nullptr);
        ++L;
    }
    if (X.launches) *X.launches += L;
}

template <int ACC, bool DET>
static void mixed_step_acc(const MixedCtx& X, int phase, cudaStream_t s) {
    const MCtx& A = *(const MCtx*)X.impl;
    if (A.cf.basis == EP_BASIS_BSMPM) mixed_step_impl<EP_BASIS_BSMPM, ACC, DET>(X, phase, s);
    else if (A.cf.basis == EP_BASIS_GIMPM) mixed_step_impl<EP_BASIS_GIMPM, ACC, DET>(X, phase, s);
    else mixed_step_impl<EP_BASIS_SMPM, ACC, DET>(X, phase, s);
}

void mixed_step(const MixedCtx& X, int phase, cudaStream_t s) {
    struct PdlScope {
        bool old;
        explicit PdlScope(bool off) : old(g_pdl_suspended) { g_pdl_suspended = off || old; }
        ~PdlScope() {
            g_pdl_suspended = old;
            g_pdl_skip_next = false;
        }
    } pdl_scope(X.prof && X.prof->on);
    const MCtx& A = *(const MCtx*)X.impl;
    if (A.g.dim == 3) {
        const int b = A.cf.basis;
        auto run = [&](auto acc, auto det) {
            constexpr int AC = decltype(acc)::value;
            constexpr bool DT = decltype(det)::value;
            if (b == EP_BASIS_BSMPM) mixed_step3_impl<EP_BASIS_BSMPM, AC, DT>(X, phase, s);
            else if (b == EP_BASIS_GIMPM) mixed_step3_impl<EP_BASIS_GIMPM, AC, DT>(X, phase, s);
            else mixed_step3_impl<EP_BASIS_SMPM, AC, DT>(X, phase, s);
        };
        using I0 = std::integral_constant<int, 0>;
        using I1 = std::integral_constant<int, 1>;
        using BF = std::integral_constant<bool, false>;
        using BT = std::integral_constant<bool, true>;
        if (A.acc == 0) {
            if (A.cf.det) run(I0(), BT());
            else run(I0(), BF());
        } else {
            if (A.cf.det) run(I1(), BT());
            else run(I1(), BF());
        }
        return;
    }
    if (A.cf.det) {
        if (A.acc == 0) mixed_step_acc<0, true>(X, phase, s);
        else mixed_step_acc<1, true>(X, phase, s);
    } else {
        if (A.acc == 0) mixed_step_acc<0, false>(X, phase, s);
        else mixed_step_acc<1, false>(X, phase, s);
    }
}

void launch_mixed_scan(const MixedCtx& X, cudaStream_t s) { mixed_scan(*(const MCtx*)X.impl, 0, X.scan_in, s); }

void mixed_initial_scan(const MixedCtx& X, cudaStream_t s) { mixed_scan(*(const MCtx*)X.impl, 1, X.scan_in, s); }

void mixed_import(const MixedCtx& X, const P64& Q, cudaStream_t s, uint64_t mask) {
    const MCtx& A = *(const MCtx*)X.impl;
    const int np = A.P.np;
    if (np > 0) km_import<<<(np + 255) / 256, 256, 0, s>>>(A, Q, mask);
    // initial cell lists for the current parity
    cudaMemsetAsync(X.sort_zero, 0, X.sort_zero_bytes, s);
    if (np > 0) km_bin0<<<(np + 255) / 256, 256, 0, s>>>(A, Q);
    mixed_initial_scan(X, s);
    if (np > 0) km_place0<<<(np + 255) / 256, 256, 0, s>>>(A);
    if (A.cf.det) km_sort_cells<<<(A.g.ncell + 255) / 256, 256, 0, s>>>(A, 1);
}

void mixed_import_host(const MixedCtx& X, const HostAoS& H, uint64_t mask, cudaStream_t s, bool bin) {
    const MCtx& A = *(const MCtx*)X.impl;
    const int np = A.P.np;
    if (!bin) {
        // beside a running step: one block per SM still keeps the host link busy
        const int nb = std::min((np + XH_BS - 1) / XH_BS, sm_count());
        if (np > 0 && mask) km_import_host<<<nb, XH_BS, 0, s>>>(A, H, mask, 0);
        return;
    }
    cudaMemsetAsync(X.sort_zero, 0, X.sort_zero_bytes, s);
    if (np > 0) km_import_host<<<(np + XH_BS - 1) / XH_BS, XH_BS, 0, s>>>(A, H, mask, 1);
    mixed_initial_scan(X, s);
    if (np > 0) km_place0<<<(np + 255) / 256, 256, 0, s>>>(A);
    if (A.cf.det) km_sort_cells<<<(A.g.ncell + 255) / 256, 256, 0, s>>>(A, 1);
}

void mixed_export_host(const MixedCtx& X, const HostAoS& H, uint64_t mask, cudaStream_t s, int par) {
    const MCtx& A = *(const MCtx*)X.impl;
    const int np = A.P.np;
    // par >= 0 runs beside the rest of a step: one block per SM
    const int nb = par >= 0 ? std::min((np + XH_BS - 1) / XH_BS, sm_count()) : (np + XH_BS - 1) / XH_BS;
    if (np > 0 && mask) km_export_host<<<nb, XH_BS, 0, s>>>(A, H, mask, par);
}

void mixed_export(const MixedCtx& X, const P64& Q, const N64& QN, cudaStream_t s, bool need_eps, uint64_t mask,
                  bool nodes) {
    const MCtx& A = *(const MCtx*)X.impl;
    const int np = A.P.np;
    if (np > 0 && mask) km_export<<<(np + 255) / 256, 256, 0, s>>>(A, Q, need_eps ? 1 : 0, mask);
    if (nodes) km_export_nodes<<<(A.g.nnode + 255) / 256, 256, 0, s>>>(A, QN);
}

// host-side construction of the device context
size_t mixed_ctx_size() { return sizeof(MCtx); }

void mixed_ctx_init(void* mem, const Cfg& cf, const Geo& g, Ctl* ctl, const PM& P, const NM& N, const SM& S,
                    const double* Del, const double* Cmp, double Kc, double Gc, double Hp, double c, int acc) {
    MCtx* A = (MCtx*)mem;
    A->cf = cf;
    A->g = g;
    A->ctl = ctl;
    A->P = P;
    A->N = N;
    A->S = S;
    const int ns = g.dim == 2 ? 3 : 6;
    for (int i = 0; i < 36; ++i) {
        A->Del[i] = i < ns * ns ? (float)Del[i] : 0.f;
        A->Cmp[i] = i < ns * ns ? (float)Cmp[i] : 0.f;
        A->Deld[i] = i < ns * ns ? Del[i] : 0.0;
        A->Cmpd[i] = i < ns * ns ? Cmp[i] : 0.0;
    }
    A->Kc = (float)Kc;
    A->Gc = (float)Gc;
    A->Hp = (float)Hp;
    A->c = c;
    A->acc = acc;
    A->Kd = Kc;
    A->Gd = Gc;
    for (int i = 0; i < 36; ++i) A->DelLU[i] = A->Deld[i];
    if (ns == 3) lu_factor<3>(A->DelLU, A->piv);
    else lu_factor<6>(A->DelLU, A->piv);
    A->l2g = (float)(Del[1] / (Del[0] - Del[1]));   // λ / (2G): Del(2,1) = λ, Del(1,1) = λ + 2G
    A->rmode = EP_RMAP_EXACT;
    A->rx = A->ry = A->raux = nullptr;
    A->rpt = A->rcount = nullptr;
    A->fbcount = A->fblist = nullptr;
    A->rec_count = nullptr;
    A->rec_cap = 0;
    A->part = nullptr;
    A->ptmp = nullptr;
}

void mixed_set_det(void* mem, float* part, float* ptmp) {
    MCtx* A = (MCtx*)mem;
    A->part = part;
    A->ptmp = ptmp;
}

// ---------------------------------------------------------------------------
// persistent batch (host side)
void* mixed_batch_create(const MixedCtx* const* xs, int n, std::string* why) {
    auto no = [&](const std::string& m) -> void* {
        if (why) *why = m;
        return nullptr;
    };
    if (n <= 0) return no("empty batch");
    std::vector<MCtx> host((size_t)n);
    std::vector<BInst> inst((size_t)n);
    std::vector<int> off((size_t)3 * (n + 1), 0);
    int basis = -1, acc = -1, musl = 0, lock = 0;
    for (int i = 0; i < n; ++i) {
        const MCtx& A = *(const MCtx*)xs[i]->impl;
        if (A.g.dim != 2) return no("the persistent batch kernel runs 2d instances");
        if (A.cf.cons == EP_CONS_MC || A.cf.cons == EP_CONS_CAMC)
            return no("the MC and Cam-Clay returns run on the per-instance graphs");
        if (A.cf.det || A.cf.nonloc || A.rmode != EP_RMAP_EXACT)
            return no("deterministic mode, nonlocal averaging and the learned map run on the per-instance graphs");
        if (basis < 0) {
            basis = A.cf.basis;
            acc = A.acc;
        } else if (basis != A.cf.basis || acc != A.acc) {
            return no("instances differ in basis or precision");
        }
        musl |= A.cf.musl ? 1 : 0;
        lock |= A.cf.locking ? 1 : 0;
        host[i] = A;
        inst[i].gz = (float*)xs[i]->grid_zero;
        inst[i].gzn = (long long)(xs[i]->grid_zero_bytes / sizeof(float));
        inst[i].sz = (int*)xs[i]->sort_zero;
        inst[i].szn = (long long)(xs[i]->sort_zero_bytes / sizeof(int));
    }
    BatchImpl* b = new BatchImpl();
    b->n = n;
    b->basis = basis;
    b->acc = acc;
    b->any_musl = musl;
    b->any_lock = lock;
    cudaError_t e = cudaMalloc(&b->ctx, sizeof(MCtx) * n);
    if (e == cudaSuccess) e = cudaMalloc(&b->inst, sizeof(BInst) * n);
    if (e == cudaSuccess) e = cudaMalloc(&b->off, sizeof(int) * 3 * 3 * (n + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->bar, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&b->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(b->ctx, host.data(), sizeof(MCtx) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->inst, inst.data(), sizeof(BInst) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->bar, 0, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(b->err, 0, sizeof(int));
    // virtual-block offsets per P2G tile shape: tiles of 16 / 32 / 64 cells, points and nodes by 256
    const int tiles[3] = {16, 32, 64};
    for (int t = 0; t < 3 && e == cudaSuccess; ++t) {
        for (int i = 0; i < n; ++i) {
            const MCtx& A = host[i];
            const int nT = (A.g.ncell + tiles[t] - 1) / tiles[t];
            const int nP = std::max(1, (A.P.np + 255) / 256);
            const int nN = (A.g.nnode + 255) / 256;
            off[i + 1] = off[i] + nT;
            off[(n + 1) + i + 1] = off[(n + 1) + i] + nP;
            off[2 * (n + 1) + i + 1] = off[2 * (n + 1) + i] + nN;
        }
        e = cudaMemcpy(b->off + (size_t)t * 3 * (n + 1), off.data(), sizeof(int) * 3 * (n + 1), cudaMemcpyHostToDevice);
        b->nblk[t][0] = off[n];
        b->nblk[t][1] = off[(n + 1) + n];
        b->nblk[t][2] = off[2 * (n + 1) + n];
        int dev = 0, sms = 0, per = 0;
        if (e == cudaSuccess) e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_kernel(basis, acc, tiles[t]), 256, 0);
        b->grid[t] = std::max(1, per) * sms;
    }
    if (e != cudaSuccess) {
        if (why) *why = std::string("persistent batch: ") + cudaGetErrorString(e);
        cudaGetLastError();
        mixed_batch_destroy(b);
        return nullptr;
    }
    return b;
}

void mixed_batch_destroy(void* p) {
    BatchImpl* b = (BatchImpl*)p;
    if (!b) return;
    cudaFree(b->ctx);
    cudaFree(b->inst);
    cudaFree(b->off);
    cudaFree(b->bar);
    cudaFree(b->err);
    delete b;
}

static BatchArgs batch_args(const BatchImpl* b, int plastic, int steps, int tile, int keep_ctl) {
    const int t = tile == 16 ? 0 : (tile == 32 ? 1 : 2);
    BatchArgs a;
    a.ctx = b->ctx;
    a.inst = b->inst;
    a.n = b->n;
    a.off = b->off + (size_t)t * 3 * (b->n + 1);
    a.steps = steps;
    a.plastic_phase = plastic;
    a.any_musl = b->any_musl;
    a.any_lock = b->any_lock;
    a.keep_ctl = keep_ctl;
    a.bar = b->bar;
    a.err = b->err;
    return a;
}

// graph of one persistent launch: barrier words reset, the cooperative kernel, the flags gather
cudaError_t mixed_batch_graph(void* p, int plastic, int steps, int tile, int* dflags, cudaGraph_t g) {
    BatchImpl* b = (BatchImpl*)p;
    const int t = tile == 16 ? 0 : (tile == 32 ? 1 : 2);
    cudaGraphNode_t ms, kn, fl;
    cudaMemsetParams mp{};
    mp.dst = b->bar;
    mp.value = 0;
    mp.elementSize = 4;
    mp.width = 2;
    mp.height = 1;
    mp.pitch = 0;
    cudaError_t e = cudaGraphAddMemsetNode(&ms, g, nullptr, 0, &mp);
    BatchArgs a = batch_args(b, plastic, steps, tile, 0);
    void* args[] = {(void*)&a};
    cudaKernelNodeParams kp{};
    kp.func = (void*)batch_kernel(b->basis, b->acc, tile);
    kp.gridDim = dim3(b->grid[t]);
    kp.blockDim = dim3(256);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    if (e == cudaSuccess) e = cudaGraphAddKernelNode(&kn, g, &ms, 1, &kp);
    if (e == cudaSuccess) {
        cudaLaunchAttributeValue v{};
        v.cooperative = 1;
        e = cudaGraphKernelNodeSetAttribute(kn, cudaLaunchAttributeCooperative, &v);
    }
    const MCtx* cx = b->ctx;
    int n = b->n;
    const int* be = b->err;
    void* fargs[] = {(void*)&cx, (void*)&n, (void*)&be, (void*)&dflags};
    cudaKernelNodeParams fp{};
    fp.func = (void*)km_batch_flags;
    fp.gridDim = dim3((n + 127) / 128);
    fp.blockDim = dim3(128);
    fp.kernelParams = fargs;
    if (e == cudaSuccess) e = cudaGraphAddKernelNode(&fl, g, &kn, 1, &fp);
    return e;
}

// one eager cooperative launch (the autotuner)
cudaError_t mixed_batch_launch(void* p, int plastic, int steps, int tile, int keep_ctl, cudaStream_t s) {
    BatchImpl* b = (BatchImpl*)p;
    const int t = tile == 16 ? 0 : (tile == 32 ? 1 : 2);
    cudaError_t e = cudaMemsetAsync(b->bar, 0, 2 * sizeof(unsigned), s);
    BatchArgs a = batch_args(b, plastic, steps, tile, keep_ctl);
    void* args[] = {(void*)&a};
    if (e == cudaSuccess)
        e = cudaLaunchCooperativeKernel(batch_kernel(b->basis, b->acc, tile), dim3(b->grid[t]), dim3(256), args, 0, s);
    return e;
}

// the phase-kernel scheme: `steps` steps of every instance as phase kernels on stream s (captured
// into the batch graph by the caller, or launched eagerly by the autotuner)
void mixed_batch_phase_steps(void* p, int plastic, int steps, int tile, int keep_ctl, cudaStream_t s) {
    BatchImpl* b = (BatchImpl*)p;
    const int t = tile == 16 ? 0 : (tile == 32 ? 1 : 2);
    const BatchArgs a = batch_args(b, plastic, steps, tile, keep_ctl);
    const int* nb = b->nblk[t];
#define EP_BPS(BS, AC)                                                      \
    if (tile == 16) batch_phase_steps_t<BS, AC, 16>(a, nb, steps, s);       \
    else if (tile == 32) batch_phase_steps_t<BS, AC, 32>(a, nb, steps, s);  \
    else batch_phase_steps_t<BS, AC, 64>(a, nb, steps, s)
    if (b->basis == EP_BASIS_BSMPM) {
        if (b->acc) { EP_BPS(EP_BASIS_BSMPM, 1); } else { EP_BPS(EP_BASIS_BSMPM, 0); }
    } else if (b->basis == EP_BASIS_GIMPM) {
        if (b->acc) { EP_BPS(EP_BASIS_GIMPM, 1); } else { EP_BPS(EP_BASIS_GIMPM, 0); }
    } else {
        if (b->acc) { EP_BPS(EP_BASIS_SMPM, 1); } else { EP_BPS(EP_BASIS_SMPM, 0); }
    }
#undef EP_BPS
}

void mixed_batch_flags(void* p, int* dflags, cudaStream_t s) {
    BatchImpl* b = (BatchImpl*)p;
    km_batch_flags<<<(b->n + 127) / 128, 128, 0, s>>>(b->ctx, b->n, b->err, dflags);
}

int mixed_batch_error(void* p) {
    BatchImpl* b = (BatchImpl*)p;
    int v = 0;
    if (cudaMemcpy(&v, b->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
    return v;
}

void mixed_set_rmap(void* mem, const RmapBufs& b) {
    MCtx* A = (MCtx*)mem;
    A->rmode = b.mode;
    A->rx = b.rx;
    A->ry = b.ry;
    A->raux = b.raux;
    A->rpt = b.rpt;
    A->rcount = b.rcount;
    A->fbcount = b.fbcount;
    A->fblist = b.fblist;
    A->rec_count = b.rec_count;
    A->rec_cap = b.rec_cap;
}

}  // namespace ep
