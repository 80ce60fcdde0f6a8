// ep_mixed.cuh -- device data of the mixed-precision steps.
//
// Points: positions as FP32 offsets from the left node of the point's cell
// (the cell itself is implicit in the per-step cell lists), velocities,
// stresses and material constants in FP32.  The accumulated state -- the
// deformation gradient F, the elastic left Cauchy-Green tensor b_e and the
// accumulated plastic strain -- is either FP64 (precision "mixed") or a
// double-float pair of FP32 values hi + lo (precision "mixed_df"); only one
// of the two storages is allocated.  Offsets and cell lists are
// double-buffered: a step reads the buffer Ctl::parity and writes the other
// one, and the parity flips at the end of every executed step.
#pragma once

#include "ep_dev.cuh"

namespace ep {

struct PM {
    int np;
    float* dx[2][3];   // [parity][direction] x - x_node(e), e = the point's cell
    float* v[3];
    double* Fd[9];     // F, column-major D x D (FP64 storage)
    float* Fh[9];      // F as hi + lo FP32 pair (double-float storage)
    float* Fl[9];
    double* bd[6];     // b_e symmetric: 2d (11, 22, 12)
    float* bh[6];
    float* bl[6];
    double* ep1d;      // accumulated plastic strain ϵpII[1]
    float* ep1h;
    float* ep1l;
    float* tau[6];     // Kirchhoff (finite) or Cauchy (infinitesimal) stress, Voigt
    float* ep2;        // nonlocal ϵpII[2]
    float* dlam;
    float *c0, *cr, *tphi, *sphi, *cphi;
    float* mp;         // ρΩ of the point (finite: ρ0Ω0)
    float* Om0;
    float* Om;         // current volume (infinitesimal: J Ω0)
    float* rho;        // density (infinitesimal: stays at its uploaded value, deform.jl:25-44)
    float* l[3];       // GIMP half lengths
    float* l0[3];      // GIMP initial half lengths (domain updates relative to them, domain.jl:1-52)
    float* dv[9];      // TPIC: velocity gradient of the previous step
    int* p2e_next;     // cell of the position written by the last G2P
    int* pcell[2];     // [parity] cell of each point (nonlocal averaging: the cell at the step start)
    float4* gv;        // 2d F-bar: ∇v (xx, zx, xz, zz) of each list slot, from the F-bar pass for km_cons
    double* epv;       // ϵpV, FP64 (read and written by the Cam-Clay return only)
};

struct NM {
    float* m;
    float *p[3], *f[3], *a[3], *v[3], *pm[3], *vm[3];
    float* dJacc;      // Σ N m δJ
    float* dJn;        // nodal δJ = ΔJ_n - 1
    // 2d: the values the point kernels gather, packed per node so that each of the 16 stencil
    // nodes is one 16-byte load: (v_x, v_z, a_x, a_z) after the grid update, and (the velocity
    // ∇v is taken of (v or the mUSL v), ΔJ numerator, its scale) for the F-bar and constitutive
    // kernels: the nodal δJ is z·w, either (Σ N m δJ, 1/m) when the F-bar pass adds into z, or
    // (δJ_n, 1) when km_dJn forms it
    float4* va4;
    float4* vg4;
};

// the single-pass scan of the next-step cell counts (km_vmusl_scan): tiles of MSCAN_TILE cells,
// each publishing its aggregate / inclusive prefix in one 64-bit status word
constexpr int MSCAN_TILE = 4096;
inline int scan_tiles(int ncell) { return (ncell + MSCAN_TILE - 1) / MSCAN_TILE; }

struct SM {
    int* count[2];
    int* start[2];     // ncell + 1 each
    int* list[2];      // point ids grouped by cell
    int* cellof[2];    // cell of each list slot
    int* cursor;
    int* scan_tmp;
    // zeroed with the counts at every step start: [0] the scan's tile ticket, [1] constitutive blocks
    // done (the last one flips the parity), then one status word per scan tile
    int* sync;
    unsigned long long* scan_status;
};

}  // namespace ep
