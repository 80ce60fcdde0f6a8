/*
 * epgpu.h -- C ABI of the GB300 explicit MPM step for ElastoPlasm.jl.
 *
 * The library replaces the body of the reference's time loop: one call of
 * `shpfun(mpts,mesh,instr); mapsto(mpts,mesh,g,dt,instr); elasto|elastoplast(...)`
 * (src/home/program/workflow/worflow.jl:34-36 and 80-82) and, for whole
 * checkpoint windows, the `while T > time.t[1]` loop around it
 * (worflow.jl:27-39, 73-85).  The kernels it runs are selected by the same
 * switches that build the reference's kernel table `instr.cairn`
 * (src/home/api/kwargser.jl:49-60; require.jl:34-88).
 *
 * Conventions (mirroring the Julia side, which calls this through `ccall`):
 *  - host arrays are caller-owned and column-major, exactly the `Point`/`Mesh`
 *    fields of src/boot/needs/types.jl:38-168 (e.g. `x` is dim x nmp, stored
 *    point by point); node and element ids are 1-based Int64, 0 = none;
 *  - the library keeps its own device copy (structure of arrays) between
 *    `epgpu_upload` and `epgpu_download`;
 *  - every call returns an `ep_status`; no exception or signal crosses the
 *    ABI; `epgpu_last_error` gives the message of the last failure;
 *  - a handle is used by one host thread at a time and owns one CUDA stream.
 */
#ifndef EPGPU_H
#define EPGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EPGPU_ABI_VERSION 1

typedef enum ep_status {
    EP_OK = 0,
    EP_ERR_ARG = 1,              /* null pointer, bad size or enum value */
    EP_ERR_UNSUPPORTED = 2,      /* switch combination not built; the reference throws
                                    ArgumentError (shpfun.jl:50, mapsto.jl:44, plast.jl:31) */
    EP_ERR_NONFINITE = 3,        /* NaN/Inf found in the particle state after a step */
    EP_ERR_TIMEOUT = 5,          /* a bounded device wait gave up */
    EP_ERR_CUDA = 6,             /* CUDA runtime failure */
    EP_ERR_INVALID_POSITION = 7, /* B-spline node outside its boundary table: the
                                    reference's error("Invalid position") (bsmpm.jl:75) */
    EP_ERR_NOMEM = 8,
    EP_ERR_STATE = 9,            /* calls out of order (step before upload, ...) */
    EP_ERR_NONCONVERGED = 10     /* a return map exceeded its iteration limit (the reference
                                    throws "CPA: η_it>...", MCRetMap.jl:38-41) */
} ep_status;

/* instr.basis.which (require.jl:39) */
enum { EP_BASIS_BSMPM = 0, EP_BASIS_GIMPM = 1, EP_BASIS_SMPM = 2 };
/* instr.basis.how: GIMP domain update (update.jl:7-28) */
enum { EP_HOW_NONE = 0, EP_HOW_UNDEFORMED = 1, EP_HOW_DETFIJ = 2, EP_HOW_FII = 3, EP_HOW_UII = 4,
       EP_HOW_DETDFIJ = 5, EP_HOW_DFII = 6, EP_HOW_DUII = 7 };
/* instr.fwrk.deform / trsfr (require.jl:44-45) */
enum { EP_DEFORM_FINITE = 0, EP_DEFORM_INFINITESIMAL = 1 };
enum { EP_TRSFR_STD = 0, EP_TRSFR_TPIC = 1, EP_TRSFR_APIC = 2 };
/* instr.plast.constitutive (require.jl:68; "MC" and "camC" are the names plast.jl:14,28 dispatches on) */
enum { EP_CONS_DP = 0, EP_CONS_J2 = 1, EP_CONS_MC = 2, EP_CONS_CAMC = 3 };
/* device arithmetic: FP64 in the reference's order; FP32 transfers with FP64
 * accumulated state and isotropic log/exp; FP32 transfers with double-float
 * (FP32 pair) accumulated state */
enum { EP_PREC_FP64 = 0, EP_PREC_MIXED = 1, EP_PREC_MIXED_DF = 2 };
/* workflow phase (worflow.jl:23 elastodynamic!, :68 elastoplastic!) */
enum { EP_PHASE_ELASTODYNAMIC = 0, EP_PHASE_ELASTOPLASTIC = 1 };

/* Switches of `instr` that select kernels (require.jl:34-88). */
typedef struct ep_cfg {
    int32_t dim;           /* 2 or 3 = length(L) */
    int32_t basis;         /* EP_BASIS_*            basis.which */
    int32_t how;           /* EP_HOW_*              basis.how (gimpm only) */
    int32_t ghost;         /* basis.ghost (mesh already built with it; informative) */
    int32_t deform;        /* EP_DEFORM_*           fwrk.deform */
    int32_t trsfr;         /* EP_TRSFR_*            fwrk.trsfr */
    double  C_pf;          /* fwrk.C_pf: FLIP fraction of the PIC/FLIP blend */
    int32_t musl;          /* fwrk.musl */
    int32_t locking;       /* fwrk.locking: F-bar volumetric locking fix */
    double  damping;       /* fwrk.damping: grid viscous damping */
    int32_t constitutive;  /* EP_CONS_*             plast.constitutive */
    int32_t nonloc;        /* nonloc.status */
    double  nonloc_ls;     /* nonloc.ls: nonlocal length scale [m] */
    int32_t precision;     /* EP_PREC_FP64 (drop-in, oracle order) | EP_PREC_MIXED | EP_PREC_MIXED_DF */
    int32_t jaumann;       /* 0: reference rate (its spin term is identically zero,
                              elast.jl:77); 1: objective Jaumann rate (not the reference) */
    int32_t deterministic; /* mixed precisions: 1 = no floating-point atomics (each cell's points
                              summed in point-id order into per-cell node partials, nodes
                              summing their cells in a fixed order): bitwise reproducible runs.
                              The FP64 step is always deterministic. */
} ep_cfg;

/* Material constants: the `cmpr` NamedTuple of setup_cmpr (setup_cmpr.jl:120-143). */
typedef struct ep_cmpr {
    double E, nu, Kc, Gc;
    double Del[36];        /* nstr x nstr elastic stiffness, column-major (nstr = 3 | 6) */
    double Hp;             /* softening/hardening modulus */
    double c0, cr;         /* peak and residual cohesion defaults (per point values in mpts) */
    double phi0, phir;
    double rho0;
    double c;              /* elastic wave speed used by the CFL step (physics.jl:21-26) */
} ep_cmpr;

/* Mesh geometry (types.jl:141-168). */
typedef struct ep_mesh_view {
    int64_t dim;
    int64_t nel[4];        /* per direction then total, as mesh.nel: [nx, (ny,) nz, total] */
    int64_t nno[4];        /* same for nodes */
    int64_t nn;            /* stencil size 4^dim */
    double  h[3];
    double  x0[3];
    const double*  x;      /* dim x nno[dim]   mesh.x */
    const double*  xB;     /* dim x 2          mesh.xB */
    const uint8_t* bcs;    /* dim x nno[dim]   mesh.bcs.status (Julia Bool) */
    const int64_t* e2n;    /* nn x nel[dim]    mesh.e2n, or NULL; checked when given */
} ep_mesh_view;

/* Nodal fields for download (types.jl:151-160). */
typedef struct ep_mesh_fields {
    double* mi;            /* nno      lumped mass */
    double* p;             /* dim x nno momentum */
    double* v;             /* dim x nno velocity */
    double* a;             /* dim x nno acceleration */
    double* oobf;          /* dim x nno out-of-balance force */
    double* dJ;            /* nno      first nno linear slots of mesh.ΔJ (volumetric.jl:8) */
} ep_mesh_fields;

/* Material-point state (types.jl:38-105); any pointer may be NULL on download. */
typedef struct ep_mpts_view {
    int64_t ndim, nmp;
    double* vmax;                                   /* dim */
    double *x, *l0, *l;                             /* dim x nmp */
    double *n0, *n, *Omega0, *Omega, *dJ, *J;       /* nmp */
    double *u, *v, *p;                              /* dim x nmp (u, p not read by the step) */
    double *rho0, *rho, *c0, *cr, *phi, *dlam;      /* nmp */
    double *epII;                                   /* 2 x nmp: accumulated, nonlocal */
    double *epV;                                    /* nmp */
    double *sig, *tau;                              /* nstr x nmp Voigt (xx,yy,[zz,yz,xz,]xy) */
    double *dvij, *duij, *dFij, *Fij, *bij, *eij, *wij, *sJij; /* dim x dim x nmp */
    int64_t *p2e;                                   /* nmp, 1-based (download only) */
    int64_t *p2n;                                   /* nn x nmp, 1-based (download only) */
    double *Bij, *Dij;                              /* dim x dim x nmp: APIC's Bᵢⱼ and Dᵢⱼ
                                                       (types.jl:82-83); read and written only
                                                       with EP_TRSFR_APIC, may be NULL */
} ep_mpts_view;

typedef struct ep_stats {
    int64_t steps;          /* MPM cycles executed since create */
    int64_t launches;       /* kernels launched since create */
    double  device_ms;      /* device time of the last epgpu_run/epgpu_step call */
    double  t;              /* simulated time after the last epgpu_run */
    int64_t plastic;        /* points with Δλ != 0 after the last step */
} ep_stats;

/* Per-kernel device time, accumulated while profiling is on (epgpu_profile). */
typedef struct ep_kernel_time {
    char    name[32];
    int64_t launches;
    double  total_ms;       /* sum of CUDA-event durations on the handle's stream */
} ep_kernel_time;

typedef struct ep_handle ep_handle;

/* Library version string. */
const char* epgpu_version(void);

/* Build a device context for `nmp` points on `mesh` with switches `cfg`
 * (replaces kwargser's kernel table, kwargser.jl:49-60, and the arrays of
 * setup_mesh/setup_mpts).  Returns EP_ERR_UNSUPPORTED for switch combinations
 * the reference rejects or this library does not build (MC in 3d, 1d; APIC in the
 * mixed precisions on meshes with h >= 2.5 in 2d or h >= 100 in 3d, where the
 * reference's D⁻¹ of p2n.jl:221-225 could differ from the identity the mixed step
 * assumes: its Dᵢⱼ is rank one, so |det D| is rounding noise below 1e-12 until then). */
ep_status epgpu_create(const ep_cfg* cfg, const ep_cmpr* cmpr, const ep_mesh_view* mesh,
                       int64_t nmp, ep_handle** out);

/* Copy the point state in (host AoS -> device SoA). */
ep_status epgpu_upload(ep_handle* h, const ep_mpts_view* mpts);

/* One MPM cycle with the caller's dt and gravity g[dim]: shpfun + mapsto +
 * elasto (phase 0) or elastoplast (phase 1) (worflow.jl:34-36, 80-82).
 * vmax is reset first and the new per-direction maximum |v| is returned in
 * vmax_out[dim] (the reference's mpts.vmax after n2p, n2p.jl:37). */
ep_status epgpu_step(ep_handle* h, int32_t phase, double dt, const double* g, double* vmax_out);

/* The reference's inner time loop for one checkpoint window:
 *   while T > t: dt = min(0.5 max_i h_i/(vmax_i+c), T-t); vmax = 0;
 *                g = phase 0 ? [0..,-9.81 t/tg] (t <= tg) : [0..,-9.81];
 *                step; t += dt
 * (physics.jl:21-26, 80-90; worflow.jl:28-39, 74-85).  The loop runs on the
 * device in CUDA graphs; *t_inout is read and written back.  nsteps_out may be NULL. */
ep_status epgpu_run(ep_handle* h, int32_t phase, double T, double tg, double* t_inout,
                    int64_t* nsteps_out);

/* Called after each checkpoint window of epgpu_run_checkpoints with the window's index k (into the
 * sorted list) and the simulated time reached.  The handle is idle during the call: the callback may
 * download fields (epgpu_download, epgpu_fields, ...) the way savlot reads the Point at a checkpoint.
 * Return 0 to go on, anything else to stop after this window. */
typedef int32_t (*ep_checkpoint_cb)(ep_handle* h, int32_t k, double t, void* user);

/* One phase of the reference's workflow over a whole checkpoint list (elastodynamic!/elastoplastic!,
 * worflow.jl:23-47 and 68-93): the list is sorted ascending (worflow.jl:24,69 sort the collected
 * range), then for each T the window `while T > t` runs as epgpu_run does, and cb (may be NULL) is
 * called in place of savlot (worflow.jl:41,87).  Windows whose T <= t take no step, as in the
 * reference's while loop, but their callback is still called.  *t_inout is read and written back;
 * nsteps_out (may be NULL) receives the steps taken over all windows. */
ep_status epgpu_run_checkpoints(ep_handle* h, int32_t phase, const double* checkpoints, int32_t ncheck,
                                double tg, double* t_inout, ep_checkpoint_cb cb, void* user,
                                int64_t* nsteps_out);

/* Copy the point state out (device SoA -> host AoS); NULL fields are skipped. */
ep_status epgpu_download(ep_handle* h, ep_mpts_view* mpts);

/* ---- Moving only some point fields ------------------------------------------
 * One bit per array of ep_mpts_view.  A host that keeps the library's device state between steps
 * (the reference's time loop calls shpfun/mapsto/elastoplast on the same Point every step,
 * worflow.jl:34-36, 80-82) needs to move only what changed: the state the step reads and changes,
 * epgpu_fields_read(h) & epgpu_fields_changed(h), and nothing of the material constants after the
 * first upload. */
#define EP_MPTS_X      (1ull << 0)
#define EP_MPTS_L0     (1ull << 1)
#define EP_MPTS_L      (1ull << 2)
#define EP_MPTS_N0     (1ull << 3)
#define EP_MPTS_N      (1ull << 4)
#define EP_MPTS_OMEGA0 (1ull << 5)
#define EP_MPTS_OMEGA  (1ull << 6)
#define EP_MPTS_DJ     (1ull << 7)
#define EP_MPTS_J      (1ull << 8)
#define EP_MPTS_U      (1ull << 9)
#define EP_MPTS_V      (1ull << 10)
#define EP_MPTS_P      (1ull << 11)
#define EP_MPTS_RHO0   (1ull << 12)
#define EP_MPTS_RHO    (1ull << 13)
#define EP_MPTS_C0     (1ull << 14)
#define EP_MPTS_CR     (1ull << 15)
#define EP_MPTS_PHI    (1ull << 16)
#define EP_MPTS_DLAM   (1ull << 17)
#define EP_MPTS_EPII   (1ull << 18)
#define EP_MPTS_EPV    (1ull << 19)
#define EP_MPTS_SIG    (1ull << 20)
#define EP_MPTS_TAU    (1ull << 21)
#define EP_MPTS_DVIJ   (1ull << 22)
#define EP_MPTS_DUIJ   (1ull << 23)
#define EP_MPTS_DFIJ   (1ull << 24)
#define EP_MPTS_FIJ    (1ull << 25)
#define EP_MPTS_BIJ    (1ull << 26)   /* bij: the elastic left Cauchy-Green tensor b_e */
#define EP_MPTS_EIJ    (1ull << 27)
#define EP_MPTS_WIJ    (1ull << 28)
#define EP_MPTS_SJIJ   (1ull << 29)
#define EP_MPTS_APIC_B (1ull << 30)   /* Bij of APIC */
#define EP_MPTS_APIC_D (1ull << 31)   /* Dij of APIC */
#define EP_MPTS_ALL    ((1ull << 32) - 1ull)

/* The arrays a step of this handle reads (its switches and precision decide). */
uint64_t epgpu_fields_read(const ep_handle* h);
/* The arrays a step of this handle may change (state and the outputs derived from it). */
uint64_t epgpu_fields_changed(const ep_handle* h);

/* epgpu_upload of the arrays in `mask` only; every one of them must be non-NULL in the view.  The
 * other arrays keep their device values.  Every array in epgpu_fields_read(h) must have been
 * uploaded at least once (by this call or an earlier upload), else EP_ERR_ARG names the missing ones. */
ep_status epgpu_upload_fields(ep_handle* h, const ep_mpts_view* mpts, uint64_t mask);

/* epgpu_download of the arrays in `mask` only (each must be non-NULL in the view); vmax is written
 * when the view's vmax is non-NULL.  The mixed precisions form the log strain ϵ only when EIJ is asked. */
ep_status epgpu_download_fields(ep_handle* h, ep_mpts_view* mpts, uint64_t mask);

/* One body of a host-driven time loop in one call: epgpu_upload_fields(mpts, mask_in), epgpu_step(phase,
 * dt, g, vmax_out), epgpu_download_fields(mpts, mask_out) (worflow.jl:34-36 / 80-82 with the Point moved
 * in and out around it).  With the mixed precisions, mapped page-locked arrays and masks the direct
 * transfers handle, the three run on the device as one graph with one synchronisation at the end (F,
 * b_e, ϵpII and Δλ go up, and x and v come down, on a second stream beside the step; the graph is kept
 * while the phase, the masks and the array addresses stay the same); otherwise the three calls run in
 * turn.  The host arrays must not change during the call.  Errors are those of the three calls. */
ep_status epgpu_step_fields(ep_handle* h, ep_mpts_view* mpts, uint64_t mask_in, int32_t phase, double dt,
                            const double* g, uint64_t mask_out, double* vmax_out);

/* Copy the nodal fields of the last step out; NULL fields are skipped. */
ep_status epgpu_download_mesh(ep_handle* h, ep_mesh_fields* f);

/* The per-point plot fields of savlot (utils/savlot.jl:20-34 -> what_plot_field, utils/plot.jl:27-135),
 * evaluated on the device from the current state in FP64, so that a checkpoint moves only the fields
 * asked for instead of the whole state.  `what` is a mask of EP_FIELD_* bits; `out` receives one
 * row of np values per set bit, in bit order (row-major, popcount(what) x np).  The formulas and
 * their operation order are plot.jl's: */
#define EP_FIELD_P     (1u << 0)   /* -(σxx+σyy)/2/1e3 in 2d, -(σxx+σyy+σzz)/3/1e3 in 3d [kPa] (:28-35) */
#define EP_FIELD_SIGXX (1u << 1)   /* σxx/1e3 [kPa] (:43-44) */
#define EP_FIELD_EPSXX (1u << 2)   /* ϵ[1,1] (:53-54) */
#define EP_FIELD_EPII  (1u << 3)   /* ϵpII[1,:] (:63-64) */
#define EP_FIELD_EPV   (1u << 4)   /* ϵpV (:73-74) */
#define EP_FIELD_DU    (1u << 5)   /* sqrt(u[1]^2 + u[2]^2), also in 3d (:83-84) */
#define EP_FIELD_COH0  (1u << 6)   /* c0/1e3 [kPa] (:99-100) */
#define EP_FIELD_PHI0  (1u << 7)   /* ϕ (:106-107) */
#define EP_FIELD_N     (1u << 8)   /* n; plot.jl shows mpts.n for both "n0" and "n" (:112-123) */
#define EP_FIELD_J     (1u << 9)   /* J (:124-125) */
#define EP_FIELD_MS    (1u << 10)  /* ρ Ω (:130-131) */
#define EP_FIELD_X     (1u << 11)  /* the horizontal plot coordinate x[1,:] (:143-147) */
#define EP_FIELD_Z     (1u << 12)  /* the vertical plot coordinate: x[2,:] in 2d, x[3,:] in 3d */
#define EP_FIELD_ALL   ((1u << 13) - 1u)
/* z0 (:93-94) is a set-up constant the library does not hold; the caller's mpts.z0 serves. */
ep_status epgpu_fields(ep_handle* h, uint32_t what, double* out);

ep_status epgpu_stats(ep_handle* h, ep_stats* out);

/* Conservation sums of the current state, in FP64 with fixed-order reductions (the same state
 * gives the same bits).  Point sums use the masses ρΩ of the scatter (p2n.jl:71-75) and the
 * velocities after G2P (n2p.jl:14-40); node sums are the last step's P2G mass and the nodal
 * momentum the step left (the mUSL momentum with musl, augm.jl:13-25).  The elastic energy is
 * ½ τ·Del⁻¹τ per unit reference volume times Ω0 in finite strain (Kirchhoff τ with the log strain
 * it came from), ½ σ·Del⁻¹σ times Ω in infinitesimal strain.  The reference has no such sums; its
 * tests check mass conservation of the P2G (test/testset). */
typedef struct ep_conservation {
    double mass;               /* Σ_p ρ_p Ω_p */
    double momentum[3];        /* Σ_p ρ_p Ω_p v_p */
    double kinetic;            /* ½ Σ_p ρ_p Ω_p |v_p|² */
    double elastic;            /* Σ_p ½ τ·Del⁻¹τ Ω0 (finite) | ½ σ·Del⁻¹σ Ω (infinitesimal) */
    double mass_nodes;         /* Σ_n m_n of the last step */
    double momentum_nodes[3];  /* Σ_n p_n of the last step */
} ep_conservation;

ep_status epgpu_conservation(ep_handle* h, ep_conservation* out);

/* Per-kernel CUDA-event timers for epgpu_step (the reference only measures whole
 * kernel groups with BenchmarkTools, test/testset/test_performance.jl:1-58).
 * enable = 1 resets and starts the accumulators, 0 stops them.  While on, epgpu_step replays the
 * one-step graph captured with an event node after every kernel (programmatic launches off in it),
 * so the times hold no host launch gaps; epgpu_step_fields takes its three-call form. */
ep_status epgpu_profile(ep_handle* h, int32_t enable);

/* Copy up to `cap` accumulated kernel entries out; *count receives how many exist. */
ep_status epgpu_profile_read(ep_handle* h, ep_kernel_time* out, int32_t cap, int32_t* count);

/* Release every device resource of the handle. */
ep_status epgpu_destroy(ep_handle* h);

/* Message of the last failure on `h` (or of the last epgpu_create failure when h is NULL). */
const char* epgpu_last_error(const ep_handle* h);

/* Stand-alone particle binning (the topology kernel p2e2n_{2,3}d, tplgy.jl:43-96)
 * as a stable counting sort, on device pointers.
 *   x_dev       dim arrays of nmp doubles, direction-major (x[0..nmp), then y/z)
 *   p2e_dev     out: nmp int32, 0-based cell of each point (clamped like the reference)
 *   cell_start  out: ncell+1 int32 offsets into cell_list
 *   cell_list   out: nmp int32 point ids, grouped by cell, ascending inside a cell
 * ncell = prod(nel[0..dim)).  The call allocates its scratch (per-cell counters)
 * on the device and frees it before returning; it runs on `stream`
 * (cudaStream_t, NULL = legacy default stream) and synchronises it. */
ep_status epgpu_bin_cells(int32_t dim, const int64_t* nel, const double* h, const double* x0,
                          const double* x_dev, int64_t nmp, int32_t* p2e_dev,
                          int32_t* cell_start_dev, int32_t* cell_list_dev, void* stream);

/* Largest cell count epgpu_bin_cells_noalloc accepts (prod(nel[0..dim))). */
#define EPGPU_NOALLOC_MAX_CELLS 524288

/* epgpu_bin_cells without any device allocation.  It has no counterpart in
 * the reference: it exists for callers that must not allocate device memory
 * during the call -- a host framework whose caching allocator already owns
 * the device memory budget (CUDA.jl's pool, PyTorch), or a pipeline where
 * cudaMalloc/cudaFree would serialise the device.  The scratch (per-cell
 * counters and cursors, scan totals: about 4 MB) is one static array in
 * device memory, held by every GPU that loads the library until the process
 * exits.  Every call looks up the array's device address (cudaGetSymbolAddress)
 * in the current context, so the call stays valid after a cudaDeviceReset or a
 * re-created primary context; the first call on a device may load the
 * library's device code, so make it before any stream capture.  All calls share the array and clear what must
 * start at zero, so calls that overlap on the GPU (different streams or
 * threads at the same time) race: serialise them.  Inputs, outputs, the
 * stream and the synchronisation are as for epgpu_bin_cells; a mesh with
 * more than EPGPU_NOALLOC_MAX_CELLS cells returns EP_ERR_ARG with the reason
 * in epgpu_last_error(NULL). */
ep_status epgpu_bin_cells_noalloc(int32_t dim, const int64_t* nel, const double* h, const double* x0,
                                  const double* x_dev, int64_t nmp, int32_t* p2e_dev,
                                  int32_t* cell_start_dev, int32_t* cell_list_dev, void* stream);

/* ---- Batched ensemble -----------------------------------------------------
 * No counterpart in the reference (one slump per Julia process).  n independent
 * instances -- each its own mesh, points, switches, material and time loop --
 * advance together, by up to 16 of their own CFL steps per launch of a CUDA graph.
 * When every instance is a 2d mixed-precision step with the exact return map (no
 * deterministic mode, no nonlocal averaging) and the same basis and precision,
 * each phase of the step walks the blocks of all instances, either as one
 * persistent cooperative kernel (grid barriers between the phases; scheme 1) or as
 * one kernel per phase (scheme 2, the default).  Otherwise, or when the autotuner finds
 * it faster, (scheme 0) each instance keeps its 16-step graph and the batch graph
 * holds those graphs as independent child nodes. */
typedef struct ep_batch ep_batch;

/* cfg, cmpr, mesh, nmp: arrays of n, one entry per instance (as epgpu_create). */
ep_status epgpu_batch_create(int32_t n, const ep_cfg* cfg, const ep_cmpr* cmpr, const ep_mesh_view* mesh,
                             const int64_t* nmp, ep_batch** out);
ep_status epgpu_batch_upload(ep_batch* b, int32_t i, const ep_mpts_view* m);
ep_status epgpu_batch_download(ep_batch* b, int32_t i, ep_mpts_view* m);
/* One checkpoint window of every instance's time loop (worflow.jl:27-44 /
 * 73-85): instance i runs from t_inout[i] to T with its own dt; on return
 * t_inout[i] = T (or where an error stopped it) and nsteps_out[i] its steps. */
ep_status epgpu_batch_run(ep_batch* b, int32_t phase, double T, double tg, double* t_inout, int64_t* nsteps_out);
/* Autotuner of the mixed step: times dt = 0 steps (they leave the state unchanged)
 * of all instances with P2G tiles of 16, 32 and 64 cells per CTA -- on the instances'
 * own step graphs and, when the batch qualifies, on the persistent kernel and on the
 * phase kernels -- and keeps the fastest scheme and tile; ms_out (3) receives the
 * mean batch-step time of each tile in the chosen scheme. */
ep_status epgpu_batch_autotune(ep_batch* b, int32_t phase, int32_t* tile_out, double* ms_out);
/* The scheme the batch runs: 0 per-instance graphs, 1 persistent kernel, 2 phase kernels. */
int32_t epgpu_batch_scheme(ep_batch* b);
/* Force the scheme (0, 1, 2; EP_ERR_UNSUPPORTED when the batch does not qualify for
 * 1 or 2), or -1 back to the default. */
ep_status epgpu_batch_set_scheme(ep_batch* b, int32_t scheme);
/* The autotuner's timings (ms per batch step): ms9[3 s + k] for scheme s and the P2G
 * tile 16 / 32 / 64 (k = 0 / 1 / 2), 0 where not timed; *kernels_available: whether
 * the batch qualifies for schemes 1 and 2. */
ep_status epgpu_batch_tuning(ep_batch* b, double* ms9, int32_t* kernels_available);
/* Device time of the last epgpu_batch_run and the batch-graph launches so far. */
ep_status epgpu_batch_stats(ep_batch* b, double* device_ms, int64_t* graph_launches);
/* The handle of instance i (epgpu_stats, epgpu_set_return_map, ...); owned by the batch. */
ep_handle* epgpu_batch_instance(ep_batch* b, int32_t i);
const char* epgpu_batch_last_error(ep_batch* b);
ep_status epgpu_batch_destroy(ep_batch* b);

/* ---- Learned return map --------------------------------------------------
 * No counterpart in the reference.  A 6 -> 128 x 4 (SiLU) -> 3 MLP, BF16
 * operands with FP32 accumulation on the tensor cores, that stands in for the
 * 2d finite-strain Drucker-Prager return of the mixed-precision step
 * (elast.jl:51-54 and DP.jl:33-66, which the reference evaluates with an eigen
 * decomposition, log and exp per point).  It works in the principal frame of
 * the trial log strain, scaled by the current cohesion c (strains by
 * s = c / (2G), stresses by c).  A row of features holds EP_MLP_NX floats:
 *   x0 >= x1 the principal trial strains / s, x2 = 0 (plane strain),
 *   x3 = c / 2e4 Pa, x4 = tan(phi), x5 = tan(psi) (0), x6 = phi_n = f_s / c >= 0
 * (the scaled overstress of the trial stress), x7 unused; the network reads
 * x0..x5.  A row of outputs holds EP_MLP_NY floats (3 used): the plastic
 * correction per unit overstress, returned strains / s = x[0..2] + phi_n * y.
 * In the step, with tan(psi) = 0 the volumetric part of y is removed before use
 * (the exact return's plastic flow is then deviatoric and keeps the mean stress).
 * Parameters (FP32 master copy, EP_MLP_NPARAM floats): W1 (128 x 6), b1,
 * W2, b2, W3, b3, W4, b4 (128 x 128 each), W5 (3 x 128), b5, W row-major
 * (output x input). */
#define EP_MLP_NX 8
#define EP_MLP_NY 4
#define EP_MLP_NPARAM 50819

typedef struct ep_mlp ep_mlp;

enum {
    EP_RMAP_EXACT = 0,    /* the step's own return map (default) */
    EP_RMAP_LEARNED = 1,  /* trial-yielding points go through the network; a point whose
                             returned stress misses the yield surface by more than 1e-3 c,
                             changes the trial mean stress by more than 1e-3 c (psi = 0
                             makes the exact return keep it), swaps the principal order,
                             implies a negative plastic multiplier, or whose trial lies
                             beyond the apex (P >= c / tan(phi), where the exact map may
                             move the mean stress), is returned by the exact FP64 map */
    EP_RMAP_RECORD = 2    /* the exact map runs; (features, exact label) pairs of every
                             trial-yielding point are appended to the network's record
                             buffer until it is full */
};

/* Network with He-initialised weights from `seed`; lambda_over_2G = lambda / (2G)
 * of the material whose labels it learns (Del[0,1] / (Del[0,0] - Del[0,1])). */
ep_status epgpu_mlp_create(uint64_t seed, double lambda_over_2G, ep_mlp** out);
ep_status epgpu_mlp_destroy(ep_mlp* m);
const char* epgpu_mlp_last_error(ep_mlp* m);
ep_status epgpu_mlp_set_params(ep_mlp* m, const float* params, int64_t n);
ep_status epgpu_mlp_get_params(ep_mlp* m, float* params, int64_t n);
/* y (n x EP_MLP_NY) = network(x (n x EP_MLP_NX)), host buffers. */
ep_status epgpu_mlp_forward(ep_mlp* m, const float* x, int64_t n, float* y);
/* Device time of the forward kernel alone over n rows (zero features in the network's own buffer;
 * the work per row does not depend on the values): one untimed launch, then reps launches between
 * two CUDA events on the network's stream; *ms_per_launch = their mean.  No counterpart in the
 * reference: the measurement of the tensor-core kernel the learned return map runs in each step. */
ep_status epgpu_mlp_time(ep_mlp* m, int64_t n, int32_t reps, double* ms_per_launch);
/* Gradient of the loss sum((y - t)^2) / (3 n) over the 3 outputs, from one
 * forward and backward pass on the tensor cores; t is n x EP_MLP_NY. */
ep_status epgpu_mlp_grad(ep_mlp* m, const float* x, const float* t, int64_t n, float* grad, double* loss);
/* `iters` Adam steps (lr, beta 0.9 / 0.999) on mini-batches of `batch` rows drawn
 * with `seed` from the n rows (x, t) in host memory, or from the record buffer
 * when x is NULL.  *loss_out receives the loss of the last mini-batch.  The first
 * call on a network's initial weights (epgpu_mlp_create, not set_params) sets the
 * output bias to the mean target of the data first. */
ep_status epgpu_mlp_train(ep_mlp* m, const float* x, const float* t, int64_t n, int32_t iters, int32_t batch,
                          float lr, uint64_t seed, double* loss_out);
/* Exact FP64 labels of feature rows on the host (the reference's DP return
 * applied in the principal frame); rows that do not yield get y = 0. */
ep_status epgpu_mlp_label(const float* x, int64_t n, double lambda_over_2G, float* y);
/* (Re)allocate the record buffer for `capacity` pairs and empty it. */
ep_status epgpu_mlp_record_buffer(ep_mlp* m, int64_t capacity);
/* Pairs recorded so far (*count may exceed the capacity: only the first
 * `capacity` are kept); copies up to `cap` of them to x, t when given. */
ep_status epgpu_mlp_recorded(ep_mlp* m, int64_t* count, float* x, float* t, int64_t cap);

/* ---- Random fields -------------------------------------------------------
 * Seeded Gaussian random field at the points (cohesion fields of the scaled-up
 * slumps).  The reference's generator (utils/setup/mpts/GRF.jl:66-141) draws a
 * Gaussian-covariance field on a grid; its exponential branch is not wired in
 * (mpts_populate.jl:49-51).  This one is the randomization (spectral) method
 * evaluated at the point positions: value = max(mean + f(x), vmin) with
 * f = std / sqrt(nh) sum_k [xi_k cos(kappa_k . x) + eta_k sin(kappa_k . x)],
 * correlation rho(|dx / ell|), rho(r) = exp(-r) (exponential) or exp(-r^2)
 * (Gaussian).  The spectrum comes from one splitmix64 stream of `seed`. */
enum { EP_GRF_GAUSSIAN = 0, EP_GRF_EXPONENTIAL = 1 };
typedef struct ep_grf {
    int32_t dim;           /* 2 or 3 */
    int32_t covariance;    /* EP_GRF_* */
    int32_t nh;            /* harmonics (the reference uses 5000) */
    int32_t pad_;
    double  ell[3];        /* correlation lengths per direction */
    double  mean, std, vmin;
    uint64_t seed;
} ep_grf;

/* The harmonics of the field on the host: kappa (nh x dim, row-major), amplitudes
 * (nh x 2: xi, eta). */
ep_status epgpu_grf_spectrum(const ep_grf* g, double* kappa, double* amplitudes);
/* Field values at np points x (dim x np column-major, the layout of mpts.x),
 * evaluated on the GPU into out (np, host). */
ep_status epgpu_grf_points(const ep_grf* g, const double* x, int64_t np, double* out);

/* Failure-detection self test (no counterpart in the reference): one CTA waits on
 * an mbarrier that nothing arrives at, with the bounded wait every tensor-core
 * kernel of the library uses.  Returns EP_ERR_TIMEOUT once the wait gave up after
 * timeout_ns (the expected outcome; the context stays usable), EP_OK if it did not. */
ep_status epgpu_selftest_wait_timeout(int64_t timeout_ns);

/* Select the return map of a mixed-precision, finite-strain, Drucker-Prager
 * handle (EP_ERR_UNSUPPORTED otherwise for modes 1 and 2).  The network must
 * outlive its use by the handle. */
ep_status epgpu_set_return_map(ep_handle* h, ep_mlp* m, int32_t mode);
/* Cumulative counts since the return map was set: points returned by the
 * network, points sent to the exact fallback, pairs recorded. */
ep_status epgpu_return_map_stats(ep_handle* h, int64_t* learned, int64_t* fallback, int64_t* recorded);

#ifdef __cplusplus
}
#endif

#endif /* EPGPU_H */
