// ep_dev.cuh -- device-side data layout of the GB300 MPM step.
//
// Points live in HBM as a structure of arrays (one contiguous stream per
// component: x[0..np), then y, ...), nodes likewise; the host C-ABI transposes
// from and to the reference's column-major Julia arrays on upload/download.
// Directions are numbered like the reference's coordinate rows: 2d (x, z),
// 3d (x, y, z).  Node and cell ids follow the reference's numbering minus one:
//   2d node = iz + nno_z*ix            cell = ez + nel_z*ex
//   3d node = iz + nno_z*ix + nno_z*nno_x*iy (same for cells)
// (utils/setup/mesh/get_coords.jl:36-52, e2n.jl:36-75, tplgy.jl:49,82).
// Stencil slot s of a point in cell e has per-direction offsets o_d in 0..3,
// node index e_d-1+o_d; 2d s = o_z + 4 o_x, 3d s = o_z + 4 o_x + 16 o_y, the
// order of e2n's loops (e2n.jl:42-70).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/epgpu.h"
#include "ep_scalar.h"

namespace ep {

struct Cfg {
    int dim, basis, how, deform, trsfr, musl, locking, cons, nonloc, jaumann;
    int det;            // mixed step without floating-point atomics
    double Cpf, damping, ls;
};

struct Geo {
    int dim, nn;
    int nel[3], nno[3];
    int ncell, nnode;
    double h[3], x0[3], xB0[3], xB1[3];
    const double* ax[3];          // node coordinates per direction (bit-exact reference values)
    const signed char* cls[3];    // B-spline node class per direction node (ep_scalar.h BS_*)
    const unsigned char* bcs;     // dim x nnode Dirichlet mask, bcs[d*nnode + n]
    const int* bcw;               // the same mask as one word per node: bit d set = fixed in direction d
    int nnel[3];                  // nonlocal neighbourhood half width (e2e.jl:24)
};

struct Mat {
    double Kc, Gc, Hp, c;
    double Del[36];
    double DelLU[36];
    int piv[6];
};

// Time-loop control block, device resident: the step's dt and g live here so
// a whole checkpoint window runs inside CUDA graphs without host round trips.
struct Ctl {
    double t, dt, T, tg;
    double g[3];
    unsigned long long vmax_bits[3];  // max |v| per direction as IEEE bits (non-negative -> monotone)
    int active;                       // 0: the window is finished, every kernel returns at once
    int phase;
    long long nsteps;
    long long plastic;
    int err;                          // first error code raised by a kernel (0 = none)
    int err_info;
    int parity;                       // mixed step: which position / cell-list buffer is current
    int pad_;
    unsigned long long rm_learned;    // learned return map: points the network returned
    unsigned long long rm_fallback;   // points sent to the exact FP64 return instead
};

struct P64 {
    int np;
    double *x[3], *xo[3], *v[3], *l[3], *l0[3];
    double *n0, *n, *Om0, *Om, *dJ, *J, *rho0, *rho, *c0, *cr, *tphi, *sphi, *cphi, *dlam, *ep1, *ep2;
    double* epv;                      // ϵpV (written by the Cam-Clay return only)
    double *sig[6], *tau[6];
    double *dv[9], *dF[9], *F[9], *b[9], *eps[9], *w[9], *sJ[9];
    double *B[9], *Dm[9], *BD[9];     // APIC: Bᵢⱼ, Dᵢⱼ and the step's Bᵢⱼ D⁻¹ (scratch)
    double* SH;                       // per-direction shape table [(d*4+o)*2+c][np]
    int* p2e;                         // 0-based cell of each point
};

struct N64 {
    double* m;
    double *p[3], *oobf[3], *a[3], *v[3];
    double* dJ;
};

struct Sort {
    int* cell_count;
    int* cell_start;   // ncell + 1
    int* cell_cursor;
    int* cell_list;    // np
    int* node_count;
    int* node_start;   // nnode + 1
    int* node_cursor;
    int* node_list;    // np * nn
    int* scan_tmp;     // block sums
};

__device__ __forceinline__ void set_err(Ctl* c, int code, int info) {
    if (atomicCAS(&c->err, 0, code) == 0) c->err_info = info;
}

// Start of a step of the device time loop (worflow.jl:28-39/74-85): the window is over once t
// reaches T; dt = min(0.5 max_i h_i / (vmax_i + c), T - t) (physics.jl:21-26), vmax reset, gravity
// ramped over tg in the elastodynamic phase (physics.jl:60-90).  One thread.
__device__ __forceinline__ void ctl_begin_run(Ctl* c, int dim, double h0, double h1, double h2, double cw) {
    if (c->err) {
        c->active = 0;
        return;
    }
    if (!(c->T > c->t)) {
        c->active = 0;
        return;
    }
    double hh[3] = {h0, h1, h2};
    double cm = 0.0;
    for (int i = 0; i < dim; ++i) {
        double vm = __longlong_as_double((long long)c->vmax_bits[i]);
        double q = hh[i] / (vm + cw);
        if (i == 0 || q > cm || q != q) cm = q;
    }
    double a = 0.5 * cm, b = c->T - c->t;
    c->dt = (a < b) ? a : b;
    for (int i = 0; i < 3; ++i) c->vmax_bits[i] = 0ull;
    double G = 9.81;
    if (c->phase == EP_PHASE_ELASTODYNAMIC && c->t <= c->tg) G = 9.81 * c->t / c->tg;
    for (int i = 0; i < 3; ++i) c->g[i] = 0.0;
    c->g[dim - 1] = -G;
    c->active = 1;
    c->plastic = 0;
}

// end of an executed step: t += dt
__device__ __forceinline__ void ctl_end(Ctl* c) {
    if (!c->active) return;
    if (c->err) {
        c->active = 0;
        return;
    }
    c->t = c->t + c->dt;
    c->nsteps += 1;
}

// Element of a point, as p2e2n_{2,3}d computes it (tplgy.jl:43-96):
// e_d = clamp(fld(x_d - x0_d, h_d), 0, nel_d - 1) with Julia's exact float
// fld; the cell id is then formed in integers (same value as the reference's
// Float64 expression 1 + e_z + nel_z e_x [+ nel_z nel_x e_y], minus one).
// Returns -1 for a non-finite coordinate.
template <int D>
__device__ __forceinline__ int cell_index(const double* xp, const Geo& g, int* e) {
    for (int d = 0; d < D; ++d) {
        double f = jfld(xp[d] - g.x0[d], g.h[d]);
        if (f != f) return -1;
        double hi = (double)(g.nel[d] - 1);
        f = f < 0.0 ? 0.0 : (f > hi ? hi : f);
        e[d] = (int)f;
    }
    if (D == 2) return e[1] + g.nel[1] * e[0];
    return e[2] + g.nel[2] * e[0] + g.nel[2] * g.nel[0] * e[1];
}

// Per-direction element indices of a cell id.
template <int D>
__device__ __forceinline__ void cell_coords(int c, const Geo& g, int* e) {
    if (D == 2) {
        e[0] = c / g.nel[1];
        e[1] = c - e[0] * g.nel[1];
    } else {
        int nzx = g.nel[2] * g.nel[0];
        e[1] = c / nzx;
        int r = c - e[1] * nzx;
        e[0] = r / g.nel[2];
        e[2] = r - e[0] * g.nel[2];
    }
}

template <int D>
__device__ __forceinline__ int node_id(const int* i, const Geo& g) {
    if (D == 2) return i[1] + g.nno[1] * i[0];
    return i[2] + g.nno[2] * i[0] + g.nno[2] * g.nno[0] * i[1];
}

template <int D>
__device__ __forceinline__ void node_coords(int n, const Geo& g, int* i) {
    if (D == 2) {
        i[0] = n / g.nno[1];
        i[1] = n - i[0] * g.nno[1];
    } else {
        int nzx = g.nno[2] * g.nno[0];
        i[1] = n / nzx;
        int r = n - i[1] * nzx;
        i[0] = r / g.nno[2];
        i[2] = r - i[0] * g.nno[2];
    }
}

// stencil slot from per-direction offsets (e2n.jl loop order)
template <int D>
__device__ __forceinline__ int slot_of(const int* o) {
    if (D == 2) return o[1] + 4 * o[0];
    return o[2] + 4 * o[0] + 16 * o[1];
}

template <int D>
__device__ __forceinline__ void slot_offsets(int s, int* o) {
    if (D == 2) { o[0] = s >> 2; o[1] = s & 3; }
    else { o[1] = s >> 4; o[0] = (s >> 2) & 3; o[2] = s & 3; }
}

}  // namespace ep
