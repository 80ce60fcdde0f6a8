// ep_mixed.cuh -- device data of the mixed-precision step.
//
// Points: FP64 for the accumulated kinematic state (positions, F, b_e) and the
// accumulated plastic strain; FP32 for velocities, stresses, material
// constants and every transfer.  Positions are double-buffered (the step reads
// the positions at its start while G2P writes the new ones); the buffer in use
// is Ctl::parity, flipped at the end of each executed step.  Cell lists of the
// points (counting sort, unordered inside a cell) are double-buffered the same
// way: the step walks the lists of its start positions and builds the lists of
// the next step.
#pragma once

#include "ep_dev.cuh"

namespace ep {

struct PM {
    int np;
    double* x[2][3];   // [parity][direction]
    float* v[3];
    double* F[9];      // deformation gradient, column-major D x D
    double* b[6];      // elastic left Cauchy-Green, symmetric: 2d (11,22,12); 3d (11,22,33,23,13,12)
    float* tau[6];     // Kirchhoff stress (finite) or Cauchy stress (infinitesimal), Voigt
    double* ep1;       // accumulated plastic strain ϵpII[1]
    float* ep2;        // nonlocal ϵpII[2]
    float* dlam;
    float *c0, *cr, *tphi, *sphi, *cphi;
    float* mp;         // ρΩ of the point (finite: ρ0Ω0)
    float* Om0;
    float* Om;         // current volume (infinitesimal: J Ω0)
    float* rho;        // density (infinitesimal: stays at its uploaded value, deform.jl:25-44)
    float* l[3];       // GIMP half lengths
    float* dv[9];      // TPIC: velocity gradient of the previous step
    int* p2e_next;     // cell of the new position
};

struct NM {
    float* m;
    float *p[3], *f[3], *a[3], *v[3], *pm[3], *vm[3];
    float* dJacc;      // Σ N m δJ
    float* dJn;        // nodal δJ = ΔJ_n - 1
};

struct SM {
    int* count[2];
    int* start[2];     // ncell + 1 each
    int* list[2];
    int* cursor;
    int* scan_tmp;
};

}  // namespace ep
