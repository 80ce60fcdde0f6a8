// ep_api.cu -- the C ABI of include/epgpu.h: handle life cycle, host <->
// device transposes (Julia column-major AoS <-> device SoA), the step and the
// device-resident time loop captured in CUDA graphs.
#include <climits>
#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/epgpu.h"
#include "ep_internal.h"
#include "ep_rmap.h"

using namespace ep;

namespace {

thread_local std::string g_create_error;
constexpr int GRAPH_STEPS = 16;

struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
};

}  // namespace

// conservation sums: blocks of the fixed-order reduction and quantities per block
constexpr int SUM_BLOCKS = 512;
constexpr int SUM_Q = 10;

struct ep_handle {
    ep_cfg cfg;
    ep_cmpr cm;
    int dim = 0, nstr = 0, nn = 0;
    int np = 0, nnode = 0, ncell = 0;
    int64_t nel[4] = {0, 0, 0, 0}, nno[4] = {0, 0, 0, 0};
    cudaStream_t s = nullptr;
    std::vector<void*> allocs;
    double* pbuf = nullptr;       // point SoA
    double* nbuf = nullptr;       // node SoA
    Fp64Ctx ctx{};
    Ctl* ctl = nullptr;           // device control block
    Ctl* hctl = nullptr;          // pinned mirror
    double* stage = nullptr;      // device staging for AoS transposes
    size_t stage_n = 0;
    // upload/download: one staging slot per multi-component field (no sync between fields), the
    // fields the step never touches (u, p, ∇u, ϵpV) on the device as the caller gave them, and
    // tan/sin/cos of ϕ recomputed only when ϕ changes
    double* xfer = nullptr;
    double* pass = nullptr;
    std::vector<double> phi_cache, tphi_host;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    cudaGraph_t graph_def[2] = {nullptr, nullptr};   // kept: a batch embeds it as a child graph
    long long graph_kernels[2] = {0, 0};
    cudaGraphExec_t step_graph[2] = {nullptr, nullptr};   // one step (epgpu_step), dt and g from Ctl
    long long step_kernels[2] = {0, 0};
    // epgpu_profile: the one-step graph with an event between kernels (for the phase it was taken in),
    // the number of its marks and their names
    cudaGraphExec_t prof_graph = nullptr;
    int prof_phase = -1, prof_n = 0;
    long long prof_kernels = 0;
    std::vector<const char*> prof_names;
    int graph_gen = 0;            // bumped whenever the captured kernels' arguments change
    long long launches = 0;
    int64_t steps = 0;
    double last_ms = 0.0;
    double t = 0.0;
    bool uploaded = false;
    std::string err;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // epgpu_step_fields: the second stream of its overlapped transfers and their events (made on first use)
    cudaStream_t s2 = nullptr;
    cudaEvent_t ev_up = nullptr, ev_late = nullptr, ev_moved = nullptr, ev_dn = nullptr;
    // the whole call as one graph (uploads, step, downloads; the overlapped transfers as branches on s2),
    // kept for the configuration it was captured with: phase, masks and host array addresses
    cudaGraphExec_t fields_graph = nullptr;
    long long fields_kernels = 0;
    int fields_phase = -1;
    uint64_t fields_in = 0, fields_out = 0;
    HostAoS fields_hin{}, fields_hout{};
    Prof prof;
    bool mixed = false;
    MixedCtx mx{};
    std::vector<unsigned char> mx_impl;   // host image of the mixed kernels' argument block
    // learned return map slots (allocated on first use)
    float* rm_buf = nullptr;
    int* rm_int = nullptr;
    ep_mlp* rm_net = nullptr;
    int rm_mode = 0;
    double* sums = nullptr;       // conservation sums: per-block partials, then the totals
    uint64_t have = 0;            // EP_MPTS_* arrays uploaded at least once
    uint64_t fresh = 0;           // mixed precisions: the staging arrays (EP_MPTS_* bits) that hold the
                                  // current state (a step clears it; exports and uploads set bits)
};

void ep::set_global_error(const char* msg) { g_create_error = msg ? msg : ""; }

static double bits_to_double(unsigned long long b) {
    double v;
    std::memcpy(&v, &b, sizeof(double));
    return v;
}

static ep_status fail(ep_handle* h, ep_status st, const std::string& m) {
    if (h) h->err = m;
    else g_create_error = m;
    return st;
}

static ep_status cuda_fail(ep_handle* h, cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return fail(h, EP_ERR_CUDA, m);
}

#define CK(h, call)                                                  \
    do {                                                             \
        cudaError_t e__ = (call);                                    \
        if (e__ != cudaSuccess) return cuda_fail((h), e__, #call);   \
    } while (0)

template <class T>
static cudaError_t dalloc(ep_handle* h, T** p, size_t n) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, (n ? n : 1) * sizeof(T));
    if (e == cudaSuccess) {
        h->allocs.push_back(q);
        cudaMemset(q, 0, (n ? n : 1) * sizeof(T));
    }
    *p = (T*)q;
    return e;
}

// AoS (k x np, column-major) -> SoA block (k streams of np)
__global__ void k_aos_to_soa(const double* __restrict__ in, int k, int np, double* out) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    for (int c = 0; c < k; ++c) out[(size_t)c * np + p] = in[(size_t)c + (size_t)k * p];
}
__global__ void k_soa_to_aos(const double* __restrict__ in, int k, int np, double* out) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    for (int c = 0; c < k; ++c) out[(size_t)c + (size_t)k * p] = in[(size_t)c * np + p];
}

// point field blocks inside pbuf
enum Fld {
    F_X, F_XO, F_V, F_L, F_L0, F_N0, F_N, F_OM0, F_OM, F_DJ, F_J, F_RHO0, F_RHO, F_C0, F_CR, F_TPHI, F_SPHI, F_CPHI,
    F_DLAM, F_EP, F_SIG, F_TAU, F_DV, F_DF, F_F, F_B, F_EPS, F_W, F_SJ, F_SH, F_BIJ, F_DIJ, F_BD, F_COUNT
};

static int fld_width(Fld f, int d, int ns) {
    switch (f) {
        case F_X: case F_XO: case F_V: case F_L: case F_L0: return d;
        case F_EP: return 2;
        case F_SIG: case F_TAU: return ns;
        case F_DV: case F_DF: case F_F: case F_B: case F_EPS: case F_W: case F_SJ: case F_BIJ: case F_DIJ:
        case F_BD: return d * d;
        case F_SH: return 8 * d;
        default: return 1;
    }
}

static double* fld_ptr(ep_handle* h, Fld f) {
    size_t off = 0;
    for (int i = 0; i < (int)f; ++i) off += (size_t)fld_width((Fld)i, h->dim, h->nstr) * h->np;
    return h->pbuf + off;
}

extern "C" {

const char* epgpu_version(void) { return "epgpu 0.2 (sm_103a, FP64 oracle-order step, mixed FP32/FP64 step)"; }

const char* epgpu_last_error(const ep_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

// the captured graphs hold the kernels' argument blocks by value: dropped whenever those change
static void drop_graphs(ep_handle* h) {
    ++h->graph_gen;
    for (int i = 0; i < 2; ++i) {
        if (h->graph[i]) cudaGraphExecDestroy(h->graph[i]);
        if (h->graph_def[i]) cudaGraphDestroy(h->graph_def[i]);
        if (h->step_graph[i]) cudaGraphExecDestroy(h->step_graph[i]);
        h->graph[i] = nullptr;
        h->graph_def[i] = nullptr;
        h->step_graph[i] = nullptr;
    }
    if (h->prof_graph) cudaGraphExecDestroy(h->prof_graph);
    h->prof_graph = nullptr;
    h->prof_phase = -1;
    if (h->fields_graph) cudaGraphExecDestroy(h->fields_graph);
    h->fields_graph = nullptr;
    h->fields_phase = -1;
}

ep_status epgpu_destroy(ep_handle* h) {
    if (!h) return EP_ERR_ARG;
    drop_graphs(h);
    if (h->s) cudaStreamSynchronize(h->s);
    for (void* p : h->allocs) cudaFree(p);
    if (h->hctl) cudaFreeHost(h->hctl);
    if (h->s2) cudaStreamSynchronize(h->s2);
    for (cudaEvent_t e : {h->ev0, h->ev1, h->ev_up, h->ev_late, h->ev_moved, h->ev_dn})
        if (e) cudaEventDestroy(e);
    if (h->s2) cudaStreamDestroy(h->s2);
    if (h->s) cudaStreamDestroy(h->s);
    delete h;
    return EP_OK;
}

ep_status epgpu_create(const ep_cfg* cfg, const ep_cmpr* cmpr, const ep_mesh_view* mesh, int64_t nmp,
                       ep_handle** out) {
    g_create_error.clear();
    if (!cfg || !cmpr || !mesh || !out || nmp < 0) return fail(nullptr, EP_ERR_ARG, "null argument or nmp < 0");
    *out = nullptr;
    const int d = cfg->dim;
    if (d != 2 && d != 3) return fail(nullptr, EP_ERR_UNSUPPORTED, "only 2d and 3d steps are built");
    if (mesh->dim != d) return fail(nullptr, EP_ERR_ARG, "mesh.dim != cfg.dim");
    if (cfg->basis < 0 || cfg->basis > 2) return fail(nullptr, EP_ERR_UNSUPPORTED, "unknown basis.which");
    if (cfg->trsfr != EP_TRSFR_STD && cfg->trsfr != EP_TRSFR_TPIC && cfg->trsfr != EP_TRSFR_APIC)
        return fail(nullptr, EP_ERR_UNSUPPORTED, "unsupported transfer scheme (mapsto.jl:44)");
    if (cfg->deform != EP_DEFORM_FINITE && cfg->deform != EP_DEFORM_INFINITESIMAL)
        return fail(nullptr, EP_ERR_UNSUPPORTED, "unknown fwrk.deform");
    if (cfg->constitutive != EP_CONS_DP && cfg->constitutive != EP_CONS_J2 && cfg->constitutive != EP_CONS_MC &&
        cfg->constitutive != EP_CONS_CAMC)
        return fail(nullptr, EP_ERR_UNSUPPORTED, "InvalidReturnMapping (plast.jl:31)");
    if (cfg->constitutive == EP_CONS_MC && d != 2)
        return fail(nullptr, EP_ERR_UNSUPPORTED, "the MC return map is plane strain only (MCRetMap.jl uses sigma[1:3])");
    if (cfg->basis == EP_BASIS_GIMPM) {
        bool fin = cfg->deform == EP_DEFORM_FINITE;
        int w = cfg->how;
        bool ok = fin ? (w == EP_HOW_UNDEFORMED || w == EP_HOW_DETFIJ || w == EP_HOW_FII || w == EP_HOW_UII)
                      : (w == EP_HOW_UNDEFORMED || w == EP_HOW_DETDFIJ || w == EP_HOW_DFII || w == EP_HOW_DUII);
        if (!ok) return fail(nullptr, EP_ERR_UNSUPPORTED, "basis.how undefined for gimpm in this framework");
    }
    if (cfg->precision != EP_PREC_FP64 && cfg->precision != EP_PREC_MIXED && cfg->precision != EP_PREC_MIXED_DF)
        return fail(nullptr, EP_ERR_UNSUPPORTED, "unknown precision");
    if (cfg->nonloc && !(cfg->nonloc_ls > 0.0)) return fail(nullptr, EP_ERR_ARG, "nonloc.ls must be > 0");
    if (!mesh->x || !mesh->xB || !mesh->bcs) return fail(nullptr, EP_ERR_ARG, "mesh.x, mesh.xB and mesh.bcs are required");
    long long nnode = 1, ncell = 1;
    for (int i = 0; i < d; ++i) {
        if (mesh->nno[i] < 2 || mesh->nel[i] != mesh->nno[i] - 1 || !(mesh->h[i] > 0.0))
            return fail(nullptr, EP_ERR_ARG, "inconsistent mesh.nel/nno/h");
        nnode *= mesh->nno[i];
        ncell *= mesh->nel[i];
    }
    if (mesh->nno[d] != nnode || mesh->nel[d] != ncell) return fail(nullptr, EP_ERR_ARG, "mesh.nno/nel totals");
    if (cfg->trsfr == EP_TRSFR_APIC && cfg->precision != EP_PREC_FP64) {
        // the mixed step forms v + Bᵢⱼ δ, i.e. D⁻¹ = I (p2n.jl:221-225).  The reference's Dᵢⱼ is the
        // rank-one N δ δᵀ of one node (misc.jl:25) with entries M <= (2h)²; after the first pivot
        // its LU pivots are rounding noise (<= 7u M, then <= 14u M; u = 2^-53), so |det D| <= 7u M²
        // in 2d (< 1e-12 while h < 3) and <= 98u² M³ in 3d (< 1e-12 while h < 300).  The limits
        // below keep a margin; the FP64 step takes either branch exactly.
        const double hmax = d == 2 ? 2.5 : 100.0;
        for (int i = 0; i < d; ++i)
            if (!(mesh->h[i] < hmax))
                return fail(nullptr, EP_ERR_UNSUPPORTED,
                            d == 2 ? "apic in the mixed precisions needs h < 2.5 in 2d (D⁻¹ = I)"
                                   : "apic in the mixed precisions needs h < 100 in 3d (D⁻¹ = I)");
    }
    const long long NN = d == 2 ? 16 : 64;
    if (nnode > 16000000LL || ncell > 16000000LL || nmp * NN > (long long)INT_MAX)
        return fail(nullptr, EP_ERR_UNSUPPORTED, "mesh or point count beyond the 32-bit index range of this build");

    ep_handle* h = new ep_handle();
    h->cfg = *cfg;
    h->cm = *cmpr;
    h->dim = d;
    h->nstr = d == 2 ? 3 : 6;
    h->nn = (int)NN;
    h->np = (int)nmp;
    h->nnode = (int)nnode;
    h->ncell = (int)ncell;
    for (int i = 0; i < 4; ++i) { h->nel[i] = mesh->nel[i]; h->nno[i] = mesh->nno[i]; }

    // per-direction node coordinates, checked to form the tensor-product grid of get_coords
    std::vector<std::vector<double>> ax(d);
    auto node_of = [&](const int* i) -> long long {
        if (d == 2) return i[1] + mesh->nno[1] * (long long)i[0];
        return i[2] + mesh->nno[2] * (long long)i[0] + mesh->nno[2] * mesh->nno[0] * (long long)i[1];
    };
    for (int dd = 0; dd < d; ++dd) {
        ax[dd].resize(mesh->nno[dd]);
        for (int k = 0; k < mesh->nno[dd]; ++k) {
            int i[3] = {0, 0, 0};
            i[dd] = k;
            ax[dd][k] = mesh->x[dd + d * node_of(i)];
        }
    }
    for (long long n = 0; n < nnode; ++n) {
        int i[3];
        if (d == 2) { i[0] = (int)(n / mesh->nno[1]); i[1] = (int)(n % mesh->nno[1]); }
        else {
            long long nzx = mesh->nno[2] * mesh->nno[0];
            i[1] = (int)(n / nzx);
            long long r = n % nzx;
            i[0] = (int)(r / mesh->nno[2]);
            i[2] = (int)(r % mesh->nno[2]);
        }
        for (int dd = 0; dd < d; ++dd)
            if (mesh->x[dd + d * n] != ax[dd][i[dd]]) {
                epgpu_destroy(h);
                return fail(nullptr, EP_ERR_ARG, "mesh.x is not the structured grid of get_coords");
            }
    }
    // optional e2n check against the structured stencil (e2n.jl:20-78)
    if (mesh->e2n) {
        for (long long c = 0; c < ncell; ++c) {
            int e[3];
            if (d == 2) { e[0] = (int)(c / mesh->nel[1]); e[1] = (int)(c % mesh->nel[1]); }
            else {
                long long nzx = mesh->nel[2] * mesh->nel[0];
                e[1] = (int)(c / nzx);
                long long r = c % nzx;
                e[0] = (int)(r / mesh->nel[2]);
                e[2] = (int)(r % mesh->nel[2]);
            }
            for (int s = 0; s < NN; ++s) {
                int o[3], i[3];
                if (d == 2) { o[0] = s >> 2; o[1] = s & 3; }
                else { o[1] = s >> 4; o[0] = (s >> 2) & 3; o[2] = s & 3; }
                bool ok = true;
                for (int dd = 0; dd < d; ++dd) {
                    i[dd] = e[dd] - 1 + o[dd];
                    ok = ok && i[dd] >= 0 && i[dd] < mesh->nno[dd];
                }
                long long want = ok ? node_of(i) + 1 : 0;
                if (mesh->e2n[s + NN * c] != want) {
                    epgpu_destroy(h);
                    return fail(nullptr, EP_ERR_ARG, "mesh.e2n differs from the structured stencil");
                }
            }
        }
    }

    if (cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        epgpu_destroy(h);
        return fail(nullptr, EP_ERR_CUDA, "no CUDA device / stream");
    }
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);

    Geo& g = h->ctx.g;
    g.dim = d;
    g.nn = (int)NN;
    g.ncell = (int)ncell;
    g.nnode = (int)nnode;
    std::vector<signed char> cls;
    for (int dd = 0; dd < d; ++dd) {
        g.nel[dd] = (int)mesh->nel[dd];
        g.nno[dd] = (int)mesh->nno[dd];
        g.h[dd] = mesh->h[dd];
        g.x0[dd] = mesh->x0[dd];
        g.xB0[dd] = mesh->xB[dd];
        g.xB1[dd] = mesh->xB[dd + d];
        g.nnel[dd] = cfg->nonloc ? (int)ceil(cfg->nonloc_ls / mesh->h[dd]) : 0;
        double* axd;
        signed char* cd;
        if (dalloc(h, &axd, ax[dd].size()) != cudaSuccess || dalloc(h, &cd, ax[dd].size()) != cudaSuccess) {
            epgpu_destroy(h);
            return fail(nullptr, EP_ERR_NOMEM, "device allocation (mesh axes)");
        }
        cudaMemcpy(axd, ax[dd].data(), ax[dd].size() * sizeof(double), cudaMemcpyHostToDevice);
        cls.resize(ax[dd].size());
        for (size_t k = 0; k < ax[dd].size(); ++k) cls[k] = (signed char)bspline_class(ax[dd][k], g.xB0[dd], g.xB1[dd], g.h[dd]);
        cudaMemcpy(cd, cls.data(), cls.size(), cudaMemcpyHostToDevice);
        g.ax[dd] = axd;
        g.cls[dd] = cd;
    }
    {
        std::vector<unsigned char> b((size_t)d * nnode);
        for (long long n = 0; n < nnode; ++n)
            for (int dd = 0; dd < d; ++dd) b[(size_t)dd * nnode + n] = mesh->bcs[dd + d * n] ? 1 : 0;
        unsigned char* bd;
        if (dalloc(h, &bd, b.size()) != cudaSuccess) {
            epgpu_destroy(h);
            return fail(nullptr, EP_ERR_NOMEM, "device allocation (bcs)");
        }
        cudaMemcpy(bd, b.data(), b.size(), cudaMemcpyHostToDevice);
        g.bcs = bd;
        std::vector<int> w((size_t)nnode, 0);
        for (long long n = 0; n < nnode; ++n)
            for (int dd = 0; dd < d; ++dd) w[(size_t)n] |= (mesh->bcs[dd + d * n] ? 1 : 0) << dd;
        int* wd;
        if (dalloc(h, &wd, w.size()) != cudaSuccess) {
            epgpu_destroy(h);
            return fail(nullptr, EP_ERR_NOMEM, "device allocation (bcs)");
        }
        cudaMemcpy(wd, w.data(), w.size() * sizeof(int), cudaMemcpyHostToDevice);
        g.bcw = wd;
    }
    Cfg& cf = h->ctx.cf;
    cf.dim = d; cf.basis = cfg->basis; cf.how = cfg->how; cf.deform = cfg->deform; cf.trsfr = cfg->trsfr;
    cf.musl = cfg->musl; cf.locking = cfg->locking; cf.cons = cfg->constitutive; cf.nonloc = cfg->nonloc;
    cf.jaumann = cfg->jaumann; cf.det = cfg->deterministic != 0; cf.Cpf = cfg->C_pf; cf.damping = cfg->damping; cf.ls = cfg->nonloc_ls;
    Mat& mt = h->ctx.mt;
    mt.Kc = cmpr->Kc; mt.Gc = cmpr->Gc; mt.Hp = cmpr->Hp; mt.c = cmpr->c;
    const int ns = h->nstr;
    for (int i = 0; i < 36; ++i) { mt.Del[i] = (i < ns * ns) ? cmpr->Del[i] : 0.0; mt.DelLU[i] = mt.Del[i]; }
    if (ns == 3) lu_factor<3>(mt.DelLU, mt.piv);
    else lu_factor<6>(mt.DelLU, mt.piv);

    // point and node storage
    size_t pw = 0;
    for (int f = 0; f < F_COUNT; ++f) pw += (size_t)fld_width((Fld)f, d, ns);
    size_t nw = 1 + 4 * (size_t)d + 1;
    bool ok = dalloc(h, &h->pbuf, pw * (size_t)h->np) == cudaSuccess && dalloc(h, &h->nbuf, nw * (size_t)h->nnode) == cudaSuccess;
    size_t stage_n = std::max<size_t>((size_t)d * d * h->np, (size_t)h->nn * h->np / 2);
    stage_n = std::max<size_t>(stage_n, (size_t)d * h->nnode);
    ok = ok && dalloc(h, &h->stage, stage_n) == cudaSuccess;
    h->stage_n = stage_n;
    // staging slots of the multi-component point fields: x v l l0 (d each), ϵpII (2), σ τ (ns each),
    // ∇v ΔF F b ϵ ω σJ (d² each); pass-through u, p (d each), ∇u (d²), ϵpV (1)
    ok = ok && dalloc(h, &h->xfer, (size_t)(4 * d + 2 + 2 * ns + 9 * d * d) * h->np) == cudaSuccess;
    ok = ok && dalloc(h, &h->sums, (size_t)(SUM_BLOCKS + 1) * SUM_Q) == cudaSuccess;
    ok = ok && dalloc(h, &h->pass, (size_t)(2 * d + d * d + 1) * h->np) == cudaSuccess;
    if (ok && h->np) ok = cudaMemset(h->pass, 0, (size_t)(2 * d + d * d + 1) * h->np * sizeof(double)) == cudaSuccess;
    Sort& S = h->ctx.S;
    int ntmp = std::max(scan_tmp_ints((int)ncell), scan_tmp_ints((int)nnode));
    ok = ok && dalloc(h, &S.cell_count, ncell) == cudaSuccess && dalloc(h, &S.cell_start, ncell + 1) == cudaSuccess &&
         dalloc(h, &S.cell_cursor, ncell) == cudaSuccess && dalloc(h, &S.cell_list, h->np) == cudaSuccess &&
         dalloc(h, &S.node_count, nnode) == cudaSuccess && dalloc(h, &S.node_start, nnode + 1) == cudaSuccess &&
         dalloc(h, &S.node_cursor, nnode) == cudaSuccess && dalloc(h, &S.node_list, (size_t)NN * h->np) == cudaSuccess &&
         dalloc(h, &S.scan_tmp, ntmp) == cudaSuccess;
    int* p2e = nullptr;
    ok = ok && dalloc(h, &p2e, h->np) == cudaSuccess;
    ok = ok && dalloc(h, &h->ctl, 1) == cudaSuccess;
    if (!ok) {
        epgpu_destroy(h);
        return fail(nullptr, EP_ERR_NOMEM, "device allocation (points/nodes)");
    }
    if (cudaMallocHost((void**)&h->hctl, sizeof(Ctl)) != cudaSuccess) {
        cudaGetLastError();
        epgpu_destroy(h);
        return fail(nullptr, EP_ERR_NOMEM, "pinned allocation");
    }
    std::memset(h->hctl, 0, sizeof(Ctl));
    P64& P = h->ctx.P;
    P.np = h->np;
    for (int i = 0; i < d; ++i) {
        P.x[i] = fld_ptr(h, F_X) + (size_t)i * h->np;
        P.xo[i] = fld_ptr(h, F_XO) + (size_t)i * h->np;
        P.v[i] = fld_ptr(h, F_V) + (size_t)i * h->np;
        P.l[i] = fld_ptr(h, F_L) + (size_t)i * h->np;
        P.l0[i] = fld_ptr(h, F_L0) + (size_t)i * h->np;
    }
    P.n0 = fld_ptr(h, F_N0); P.n = fld_ptr(h, F_N); P.Om0 = fld_ptr(h, F_OM0); P.Om = fld_ptr(h, F_OM);
    P.dJ = fld_ptr(h, F_DJ); P.J = fld_ptr(h, F_J); P.rho0 = fld_ptr(h, F_RHO0); P.rho = fld_ptr(h, F_RHO);
    P.c0 = fld_ptr(h, F_C0); P.cr = fld_ptr(h, F_CR); P.tphi = fld_ptr(h, F_TPHI); P.sphi = fld_ptr(h, F_SPHI);
    P.cphi = fld_ptr(h, F_CPHI); P.dlam = fld_ptr(h, F_DLAM);
    P.ep1 = fld_ptr(h, F_EP); P.ep2 = fld_ptr(h, F_EP) + h->np;
    P.epv = h->pass + (size_t)(2 * d + d * d) * h->np;      // ϵpV in the pass-through block (u, p, ∇u, ϵpV)
    for (int k = 0; k < ns; ++k) {
        P.sig[k] = fld_ptr(h, F_SIG) + (size_t)k * h->np;
        P.tau[k] = fld_ptr(h, F_TAU) + (size_t)k * h->np;
    }
    for (int k = 0; k < d * d; ++k) {
        P.B[k] = fld_ptr(h, F_BIJ) + (size_t)k * h->np;
        P.Dm[k] = fld_ptr(h, F_DIJ) + (size_t)k * h->np;
        P.BD[k] = fld_ptr(h, F_BD) + (size_t)k * h->np;
        P.dv[k] = fld_ptr(h, F_DV) + (size_t)k * h->np;
        P.dF[k] = fld_ptr(h, F_DF) + (size_t)k * h->np;
        P.F[k] = fld_ptr(h, F_F) + (size_t)k * h->np;
        P.b[k] = fld_ptr(h, F_B) + (size_t)k * h->np;
        P.eps[k] = fld_ptr(h, F_EPS) + (size_t)k * h->np;
        P.w[k] = fld_ptr(h, F_W) + (size_t)k * h->np;
        P.sJ[k] = fld_ptr(h, F_SJ) + (size_t)k * h->np;
    }
    P.SH = fld_ptr(h, F_SH);
    P.p2e = p2e;
    N64& N = h->ctx.N;
    N.m = h->nbuf;
    for (int i = 0; i < d; ++i) {
        N.p[i] = h->nbuf + (size_t)(1 + i) * h->nnode;
        N.oobf[i] = h->nbuf + (size_t)(1 + d + i) * h->nnode;
        N.a[i] = h->nbuf + (size_t)(1 + 2 * d + i) * h->nnode;
        N.v[i] = h->nbuf + (size_t)(1 + 3 * d + i) * h->nnode;
    }
    N.dJ = h->nbuf + (size_t)(1 + 4 * d) * h->nnode;
    h->ctx.ctl = h->ctl;
    h->ctx.np = h->np;
    h->ctx.launches = &h->launches;
    if (cfg->precision == EP_PREC_MIXED || cfg->precision == EP_PREC_MIXED_DF) {
        h->mixed = true;
        const int acc = cfg->precision == EP_PREC_MIXED_DF ? 1 : 0;
        const int np = h->np;
        const int nc = (int)ncell, nn = (int)nnode;
        PM pm{};
        NM nm{};
        SM sm{};
        pm.np = np;
        // accumulated state: F (d*d), b (3 | 6), ep1 as FP64 or as FP32 pairs
        const int nsym = d == 2 ? 3 : 6;
        const size_t nacc = (size_t)(d * d + nsym + 1);
        double* pd = nullptr;
        float* pf = nullptr;
        bool ok2 = true;
        if (acc == 0) ok2 = dalloc(h, &pd, nacc * np) == cudaSuccess;
        // floats: dx[2][d], v[d], tau[nsym], 11 scalars, rho, l[d], dv[d*d], (pairs: 2*nacc)
        const size_t nflt = (size_t)np * (2 * d + d + nsym + 11 + 1 + 2 * d + d * d + (acc ? 2 * nacc : 0));
        ok2 = ok2 && dalloc(h, &pf, nflt) == cudaSuccess;
        int* ints = nullptr;
        // step-start zeroed region: counts (2 parities), cursor, sync words, scan status (8-byte words)
        const size_t nzero = (size_t)3 * nc + 4 + 1 + 2 * (size_t)scan_tiles(nc);
        const size_t nint = nzero + 2 * (size_t)(nc + 1) + 4 * (size_t)np + (size_t)np + 2 * (size_t)(nc + 1) +
                            (cfg->nonloc ? 2 * (size_t)np : 0);
        ok2 = ok2 && dalloc(h, &ints, nint) == cudaSuccess;
        float* nf = nullptr;
        const size_t nnf = (size_t)nn * (1 + 6 * d + 2);
        ok2 = ok2 && dalloc(h, &nf, nnf) == cudaSuccess;
        if (!ok2) {
            epgpu_destroy(h);
            return fail(nullptr, EP_ERR_NOMEM, "device allocation (mixed state)");
        }
        float* f = pf;
        auto take = [&](size_t n) { float* r = f; f += n * (size_t)np; return r; };
        for (int par = 0; par < 2; ++par)
            for (int i = 0; i < d; ++i) pm.dx[par][i] = take(1);
        for (int i = 0; i < d; ++i) pm.v[i] = take(1);
        for (int k = 0; k < nsym; ++k) pm.tau[k] = take(1);
        pm.ep2 = take(1); pm.dlam = take(1); pm.c0 = take(1); pm.cr = take(1); pm.tphi = take(1);
        pm.sphi = take(1); pm.cphi = take(1); pm.mp = take(1); pm.Om0 = take(1); pm.Om = take(1);
        pm.epv = h->pass + (size_t)(2 * d + d * d) * np;      // FP64 ϵpV in the pass-through block
        take(1);   // spare
        pm.rho = take(1);
        for (int i = 0; i < d; ++i) pm.l[i] = take(1);
        for (int i = 0; i < d; ++i) pm.l0[i] = take(1);
        for (int k = 0; k < d * d; ++k) pm.dv[k] = take(1);
        if (acc == 0) {
            double* q = pd;
            for (int k = 0; k < d * d; ++k) pm.Fd[k] = q + (size_t)k * np;
            q += (size_t)d * d * np;
            for (int k = 0; k < nsym; ++k) pm.bd[k] = q + (size_t)k * np;
            q += (size_t)nsym * np;
            pm.ep1d = q;
        } else {
            for (int k = 0; k < d * d; ++k) { pm.Fh[k] = take(1); pm.Fl[k] = take(1); }
            for (int k = 0; k < nsym; ++k) { pm.bh[k] = take(1); pm.bl[k] = take(1); }
            pm.ep1h = take(1);
            pm.ep1l = take(1);
        }
        int* ip = ints;
        int* sort_zero = ip;
        sm.count[0] = ip; ip += nc;
        sm.count[1] = ip; ip += nc;
        sm.cursor = ip; ip += nc;
        sm.sync = ip; ip += 4;
        if ((ip - ints) & 1) ++ip;                       // 8-byte alignment of the status words
        sm.scan_status = reinterpret_cast<unsigned long long*>(ip);
        ip += 2 * (size_t)scan_tiles(nc);
        const size_t zero_ints = (size_t)(ip - sort_zero);
        ip = sort_zero + nzero;
        sm.start[0] = ip; ip += nc + 1;
        sm.start[1] = ip; ip += nc + 1;
        sm.list[0] = ip; ip += np;
        sm.list[1] = ip; ip += np;
        sm.cellof[0] = ip; ip += np;
        sm.cellof[1] = ip; ip += np;
        pm.p2e_next = ip; ip += np;
        h->mx.scan_in = ip; ip += nc + 1;
        h->mx.scan_out = ip; ip += nc + 1;
        if (cfg->nonloc) {
            pm.pcell[0] = ip; ip += np;
            pm.pcell[1] = ip; ip += np;
        }
        sm.scan_tmp = S.scan_tmp;
        float* g0 = nf;
        nm.m = g0;
        for (int i = 0; i < d; ++i) nm.p[i] = g0 + (size_t)(1 + i) * nn;
        for (int i = 0; i < d; ++i) nm.f[i] = g0 + (size_t)(1 + d + i) * nn;
        for (int i = 0; i < d; ++i) nm.pm[i] = g0 + (size_t)(1 + 2 * d + i) * nn;
        for (int i = 0; i < d; ++i) nm.a[i] = g0 + (size_t)(1 + 3 * d + i) * nn;
        for (int i = 0; i < d; ++i) nm.v[i] = g0 + (size_t)(1 + 4 * d + i) * nn;
        for (int i = 0; i < d; ++i) nm.vm[i] = g0 + (size_t)(1 + 5 * d + i) * nn;
        nm.dJacc = g0 + (size_t)(1 + 6 * d) * nn;
        nm.dJn = g0 + (size_t)(2 + 6 * d) * nn;
        float4* pk = nullptr;
        if (d == 2 && dalloc(h, &pk, (size_t)2 * nn) != cudaSuccess) {
            epgpu_destroy(h);
            return fail(nullptr, EP_ERR_NOMEM, "device allocation (packed node values)");
        }
        nm.va4 = pk;
        nm.vg4 = pk ? pk + nn : nullptr;
        pm.gv = nullptr;
        if (d == 2 && dalloc(h, &pm.gv, (size_t)(np > 0 ? np : 1)) != cudaSuccess) {
            epgpu_destroy(h);
            return fail(nullptr, EP_ERR_NOMEM, "device allocation (per-slot velocity gradients)");
        }
        h->mx.grid_zero = g0;
        h->mx.grid_zero_bytes = sizeof(float) * (size_t)(1 + 3 * d) * nn;   // m, p, f, mUSL p
        h->mx.sort_zero = sort_zero;
        h->mx.sort_zero_bytes = sizeof(int) * zero_ints;
        // compliance (inverse of the nstr x nstr Del) for ε = Del \\ τ
        double Cmp[36], LU[36], e[6], x[6];
        int piv[6];
        for (int i = 0; i < nsym * nsym; ++i) LU[i] = cmpr->Del[i];
        if (nsym == 3) lu_factor<3>(LU, piv);
        else lu_factor<6>(LU, piv);
        for (int j = 0; j < nsym; ++j) {
            for (int i = 0; i < nsym; ++i) e[i] = (i == j) ? 1.0 : 0.0;
            if (nsym == 3) lu_solve<3>(LU, piv, e, x);
            else lu_solve<6>(LU, piv, e, x);
            for (int i = 0; i < nsym; ++i) Cmp[i + nsym * j] = x[i];
        }
        h->mx_impl.resize(mixed_ctx_size());
        mixed_ctx_init(h->mx_impl.data(), cf, g, h->ctl, pm, nm, sm, cmpr->Del, Cmp, cmpr->Kc, cmpr->Gc, cmpr->Hp,
                       cmpr->c, acc);
        h->mx.impl = h->mx_impl.data();
        h->mx.p2g_tile = 64;
        if (cf.det) {
            float *part = nullptr, *ptmp = nullptr;
            // per-cell node partials: 16 slots x (m, p, f) in 2d, 64 slots x (m, p, f) in 3d
            const size_t nslot = d == 3 ? (size_t)64 * 7 : (size_t)16 * 5;
            if (dalloc(h, &part, (size_t)nc * nslot) != cudaSuccess || dalloc(h, &ptmp, (size_t)np) != cudaSuccess) {
                epgpu_destroy(h);
                return fail(nullptr, EP_ERR_NOMEM, "device allocation (deterministic partials)");
            }
            mixed_set_det(h->mx_impl.data(), part, ptmp);
        }
        h->mx.launches = &h->launches;
        h->mx.prof = nullptr;
    }
    h->ctx.prof = nullptr;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        std::string m = std::string("create: ") + cudaGetErrorString(e);
        cudaGetLastError();
        epgpu_destroy(h);
        return fail(nullptr, EP_ERR_CUDA, m);
    }
    *out = h;
    return EP_OK;
}

// Point-field transfers.  Host fields are AoS (k components per point, column-major k x np); the
// device blocks are SoA.  A host buffer that the runtime reports as page-locked and mapped
// (cudaHostAlloc, cudaHostRegister, a pinned tensor) is read or written in place by k_xfer, one
// launch over all such fields that also transposes; any other buffer goes through the copy engine
// (multi-component fields through their slot of the staging area) and k_aos_to_soa/k_soa_to_aos.
// The host link is the bound either way; one kernel over all fields saves the per-copy setup of
// the ~30 separate copies.
constexpr int XF_MAX = 32, XF_EPT = 8, XF_BS = 256;
struct XferTab {
    const double* src[XF_MAX];
    double* dst[XF_MAX];
    long long cnt[XF_MAX];   // elements (k x np)
    int k[XF_MAX];
    int b0[XF_MAX + 1];      // first block of each field
    int n, dir;              // dir 0: host AoS -> device SoA; 1: device SoA -> host AoS
};

// XF_EPT elements per thread, all loads issued before the stores (many requests in flight on
// the host link); element j of the AoS side is component j % k of point j / k
__global__ void __launch_bounds__(XF_BS) k_xfer(const XferTab T) {
    const int b = blockIdx.x;
    int e = 0;
    while (e + 1 < T.n && T.b0[e + 1] <= b) ++e;
    const long long n = T.cnt[e], base = (long long)(b - T.b0[e]) * XF_BS * XF_EPT;
    const int k = T.k[e];
    const long long np = n / k;
    const double* __restrict__ src = T.src[e];
    double* __restrict__ dst = T.dst[e];
    double v[XF_EPT];
#pragma unroll
    for (int i = 0; i < XF_EPT; ++i) {
        const long long j = base + (long long)i * XF_BS + threadIdx.x;
        if (j < n) {
            const long long q = j / k, c = j - q * k;
            v[i] = T.dir == 0 ? src[j] : src[c * np + q];
        }
    }
#pragma unroll
    for (int i = 0; i < XF_EPT; ++i) {
        const long long j = base + (long long)i * XF_BS + threadIdx.x;
        if (j < n) {
            const long long q = j / k, c = j - q * k;
            if (T.dir == 0) dst[c * np + q] = v[i];
            else dst[j] = v[i];
        }
    }
}

// the device address of a mapped page-locked host buffer, else null (pageable memory)
static double* mapped_host(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer) ? (double*)a.devicePointer : nullptr;
}

struct XField {
    double* host;
    int k;
    double* dev;
    size_t n;
    double* stage;   // staging slot (k > 1)
};

// every point field of the view in transfer order, then the pass-through fields (u, p, ∇u, ϵpV:
// stored as given, k = 1)
static std::vector<XField> xfer_fields(ep_handle* h, const ep_mpts_view* m) {
    const int d = h->dim, ns = h->nstr;
    const size_t np = (size_t)h->np, dn = (size_t)d * np;
    std::vector<XField> f;
    size_t off = 0;
    auto add = [&](const double* host, int k, double* dev) {
        const size_t n = (size_t)k * np;
        double* st = nullptr;
        if (k > 1) {
            st = h->xfer + off;
            off += n;
        }
        if (host && n) f.push_back({const_cast<double*>(host), k, dev, n, st});
    };
    auto raw = [&](const double* host, double* dev, size_t n) {
        if (host && n) f.push_back({const_cast<double*>(host), 1, dev, n, nullptr});
    };
    add(m->x, d, fld_ptr(h, F_X)); add(m->v, d, fld_ptr(h, F_V)); add(m->l, d, fld_ptr(h, F_L));
    add(m->l0, d, fld_ptr(h, F_L0)); add(m->n0, 1, fld_ptr(h, F_N0)); add(m->n, 1, fld_ptr(h, F_N));
    add(m->Omega0, 1, fld_ptr(h, F_OM0)); add(m->Omega, 1, fld_ptr(h, F_OM)); add(m->dJ, 1, fld_ptr(h, F_DJ));
    add(m->J, 1, fld_ptr(h, F_J)); add(m->rho0, 1, fld_ptr(h, F_RHO0)); add(m->rho, 1, fld_ptr(h, F_RHO));
    add(m->c0, 1, fld_ptr(h, F_C0)); add(m->cr, 1, fld_ptr(h, F_CR)); add(m->dlam, 1, fld_ptr(h, F_DLAM));
    add(m->epII, 2, fld_ptr(h, F_EP)); add(m->sig, ns, fld_ptr(h, F_SIG)); add(m->tau, ns, fld_ptr(h, F_TAU));
    add(m->dvij, d * d, fld_ptr(h, F_DV)); add(m->dFij, d * d, fld_ptr(h, F_DF)); add(m->Fij, d * d, fld_ptr(h, F_F));
    add(m->bij, d * d, fld_ptr(h, F_B)); add(m->eij, d * d, fld_ptr(h, F_EPS)); add(m->wij, d * d, fld_ptr(h, F_W));
    add(m->sJij, d * d, fld_ptr(h, F_SJ));
    if (h->ctx.cf.trsfr == EP_TRSFR_APIC) {
        add(m->Bij, d * d, fld_ptr(h, F_BIJ));
        add(m->Dij, d * d, fld_ptr(h, F_DIJ));
    }
    raw(m->u, h->pass, dn);
    raw(m->p, h->pass + dn, dn);
    raw(m->duij, h->pass + 2 * dn, (size_t)d * dn);
    raw(m->epV, h->pass + (2 + d) * dn, np);
    return f;
}

// fields on mapped host memory -> the k_xfer table; the rest -> `rest`
static void xfer_split(std::vector<XField>& f, int dir, XferTab& T, int& nblk, std::vector<XField*>& rest) {
    T.n = 0;
    T.dir = dir;
    nblk = 0;
    for (auto& x : f) {
        double* hp = T.n < XF_MAX ? mapped_host(x.host) : nullptr;
        if (!hp) {
            rest.push_back(&x);
            continue;
        }
        T.src[T.n] = dir == 0 ? hp : x.dev;
        T.dst[T.n] = dir == 0 ? x.dev : hp;
        T.cnt[T.n] = (long long)x.n;
        T.k[T.n] = x.k;
        T.b0[T.n] = nblk;
        nblk += (int)((x.n + (size_t)XF_BS * XF_EPT - 1) / ((size_t)XF_BS * XF_EPT));
        ++T.n;
    }
    T.b0[T.n] = nblk;
}

// ---------------------------------------------------------------------------
// Field masks of ep_mpts_view (EP_MPTS_* of include/epgpu.h): which arrays a step reads and changes.
struct ViewField {
    uint64_t bit;
    double* ep_mpts_view::*ptr;
    const char* name;
};
static const ViewField VIEW_FIELDS[] = {
    {EP_MPTS_X, &ep_mpts_view::x, "x"}, {EP_MPTS_L0, &ep_mpts_view::l0, "l0"}, {EP_MPTS_L, &ep_mpts_view::l, "l"},
    {EP_MPTS_N0, &ep_mpts_view::n0, "n0"}, {EP_MPTS_N, &ep_mpts_view::n, "n"},
    {EP_MPTS_OMEGA0, &ep_mpts_view::Omega0, "Omega0"}, {EP_MPTS_OMEGA, &ep_mpts_view::Omega, "Omega"},
    {EP_MPTS_DJ, &ep_mpts_view::dJ, "dJ"}, {EP_MPTS_J, &ep_mpts_view::J, "J"}, {EP_MPTS_U, &ep_mpts_view::u, "u"},
    {EP_MPTS_V, &ep_mpts_view::v, "v"}, {EP_MPTS_P, &ep_mpts_view::p, "p"}, {EP_MPTS_RHO0, &ep_mpts_view::rho0, "rho0"},
    {EP_MPTS_RHO, &ep_mpts_view::rho, "rho"}, {EP_MPTS_C0, &ep_mpts_view::c0, "c0"}, {EP_MPTS_CR, &ep_mpts_view::cr, "cr"},
    {EP_MPTS_PHI, &ep_mpts_view::phi, "phi"}, {EP_MPTS_DLAM, &ep_mpts_view::dlam, "dlam"},
    {EP_MPTS_EPII, &ep_mpts_view::epII, "epII"}, {EP_MPTS_EPV, &ep_mpts_view::epV, "epV"},
    {EP_MPTS_SIG, &ep_mpts_view::sig, "sig"}, {EP_MPTS_TAU, &ep_mpts_view::tau, "tau"},
    {EP_MPTS_DVIJ, &ep_mpts_view::dvij, "dvij"}, {EP_MPTS_DUIJ, &ep_mpts_view::duij, "duij"},
    {EP_MPTS_DFIJ, &ep_mpts_view::dFij, "dFij"}, {EP_MPTS_FIJ, &ep_mpts_view::Fij, "Fij"},
    {EP_MPTS_BIJ, &ep_mpts_view::bij, "bij"}, {EP_MPTS_EIJ, &ep_mpts_view::eij, "eij"},
    {EP_MPTS_WIJ, &ep_mpts_view::wij, "wij"}, {EP_MPTS_SJIJ, &ep_mpts_view::sJij, "sJij"},
    {EP_MPTS_APIC_B, &ep_mpts_view::Bij, "Bij"}, {EP_MPTS_APIC_D, &ep_mpts_view::Dij, "Dij"},
};

static uint64_t view_mask(const ep_mpts_view* m) {
    uint64_t k = 0;
    for (const ViewField& f : VIEW_FIELDS)
        if (m->*f.ptr) k |= f.bit;
    return k;
}

// A direct transfer of a mixed-precision handle (mixed_import_host / mixed_export_host: one pass
// between the host arrays and the step's layout, no FP64 staging): every array of the view is one it
// moves (MIXED_DIRECT_FIELDS; an upload must hold the positions, from which it bins) and sits in
// mapped page-locked memory.  *H receives the arrays' device-accessible addresses.
static bool direct_view(ep_handle* h, const ep_mpts_view* m, bool up, HostAoS* H, uint64_t* mask) {
    if (!h->mixed || m->p2e || m->p2n || h->ctx.cf.trsfr == EP_TRSFR_APIC) return false;
    const uint64_t k = view_mask(m);
    if (!k || (k & ~MIXED_DIRECT_FIELDS) || (up && !(k & EP_MPTS_X))) return false;
    *H = HostAoS{};
    struct Src {
        double* src;
        double** dst;
    } tab[] = {{m->x, &H->x},     {m->v, &H->v},      {m->l, &H->l},         {m->Fij, &H->F},       {m->bij, &H->b},
               {m->tau, &H->tau}, {m->sig, &H->sig},  {m->epII, &H->ep},     {m->dlam, &H->dlam},   {m->dvij, &H->dv}};
    for (const Src& t : tab) {
        if (!t.src) continue;
        double* dp = mapped_host(t.src);
        if (!dp) return false;
        *t.dst = dp;
    }
    *mask = k;
    return true;
}

static std::string mask_names(uint64_t k) {
    std::string out;
    for (const ViewField& f : VIEW_FIELDS)
        if (k & f.bit) out += (out.empty() ? "" : ", ") + std::string(f.name);
    return out;
}

// What a step reads: the FP64 step's kernels read the previous state in place (ep_fp64.cu); the
// mixed steps read what km_import and km_bin0 take from the staging layout (ep_mixed.cu).
static uint64_t reads_of(const ep_handle* h) {
    const Cfg& c = h->ctx.cf;
    const bool fin = c.deform == EP_DEFORM_FINITE;
    uint64_t k = EP_MPTS_X | EP_MPTS_V | EP_MPTS_OMEGA0 | EP_MPTS_C0 | EP_MPTS_CR | EP_MPTS_PHI | EP_MPTS_DLAM |
                 EP_MPTS_EPII | EP_MPTS_FIJ | (fin ? EP_MPTS_TAU | EP_MPTS_BIJ : EP_MPTS_SIG);
    // the point mass ρΩ: the FP64 step forms it from ρ and Ω; the mixed steps from ρ0Ω0 in finite
    // strain (which keeps ρΩ = ρ0Ω0) and from the carried ρ and Ω in infinitesimal strain
    if (!h->mixed || !fin) k |= EP_MPTS_RHO | EP_MPTS_OMEGA;
    if (h->mixed && fin) k |= EP_MPTS_RHO0;
    if (c.basis == EP_BASIS_GIMPM) k |= EP_MPTS_L | EP_MPTS_L0;
    if (c.trsfr == EP_TRSFR_TPIC) k |= EP_MPTS_DVIJ;
    if (c.trsfr == EP_TRSFR_APIC) k |= EP_MPTS_APIC_B | (h->mixed ? 0ull : EP_MPTS_APIC_D);
    if (!h->mixed && fin) k |= EP_MPTS_J | EP_MPTS_RHO0 | EP_MPTS_N0;
    if (c.cons == EP_CONS_CAMC) k |= EP_MPTS_EPV;      // the Cam-Clay return reads and writes ϵpV
    return k;
}

// What a step may change: the state it carries and the outputs derived from it (u, p, ∇u and, but
// for the Cam-Clay return, ϵpV are the caller's and pass through unchanged; ρ0, Ω0, ℓ0, n0, c0, cr, ϕ
// are material constants).
static uint64_t changed_of(const ep_handle* h) {
    const Cfg& c = h->ctx.cf;
    uint64_t k = EP_MPTS_X | EP_MPTS_V | EP_MPTS_N | EP_MPTS_OMEGA | EP_MPTS_DJ | EP_MPTS_J | EP_MPTS_RHO |
                 EP_MPTS_DLAM | EP_MPTS_EPII | EP_MPTS_SIG | EP_MPTS_TAU | EP_MPTS_DVIJ | EP_MPTS_DFIJ | EP_MPTS_FIJ |
                 EP_MPTS_BIJ | EP_MPTS_EIJ | EP_MPTS_WIJ | EP_MPTS_SJIJ;
    if (c.basis == EP_BASIS_GIMPM && c.how != EP_HOW_UNDEFORMED && c.how != EP_HOW_NONE) k |= EP_MPTS_L;
    if (c.trsfr == EP_TRSFR_APIC) k |= EP_MPTS_APIC_B | EP_MPTS_APIC_D;
    if (c.cons == EP_CONS_CAMC) k |= EP_MPTS_EPV;
    return k;
}

uint64_t epgpu_fields_read(const ep_handle* h) { return h ? reads_of(h) : 0ull; }
uint64_t epgpu_fields_changed(const ep_handle* h) { return h ? changed_of(h) : 0ull; }

static ep_status upload_view(ep_handle* h, const ep_mpts_view* m);

ep_status epgpu_upload(ep_handle* h, const ep_mpts_view* m) {
    if (!h || !m) return EP_ERR_ARG;
    if (m->nmp != h->np || m->ndim != h->dim) return fail(h, EP_ERR_ARG, "mpts.nmp/ndim differ from create");
    if (!m->x || !m->v || !m->Omega0 || !m->Omega || !m->J || !m->rho0 || !m->rho || !m->c0 || !m->cr || !m->phi ||
        !m->dlam || !m->epII || !m->sig || !m->tau || !m->Fij || !m->bij || !m->l || !m->l0 || !m->n0 || !m->n ||
        !m->dJ || !m->dvij)
        return fail(h, EP_ERR_ARG, "a point field read by the step is NULL");
    // APIC's affine state is read by the step (p2n.jl:208-280): without it the device would keep
    // stale Bᵢⱼ/Dᵢⱼ from an earlier upload
    if (h->ctx.cf.trsfr == EP_TRSFR_APIC && (!m->Bij || !m->Dij))
        return fail(h, EP_ERR_ARG, "a point field read by the step is NULL (Bij/Dij with APIC)");
    return upload_view(h, m);
}

ep_status epgpu_upload_fields(ep_handle* h, const ep_mpts_view* m, uint64_t mask) {
    if (!h || !m) return EP_ERR_ARG;
    if (m->nmp != h->np || m->ndim != h->dim) return fail(h, EP_ERR_ARG, "mpts.nmp/ndim differ from create");
    if (mask & ~EP_MPTS_ALL) return fail(h, EP_ERR_ARG, "unknown bits in the field mask");
    const uint64_t given = view_mask(m);
    if (mask & ~given) return fail(h, EP_ERR_ARG, "a field in the mask is NULL: " + mask_names(mask & ~given));
    const uint64_t missing = reads_of(h) & ~(mask | h->have);
    if (missing) return fail(h, EP_ERR_ARG, "fields read by the step were never uploaded: " + mask_names(missing));
    // the arrays outside the mask keep their device values: in the mixed precisions those live in the
    // step's own layout and the import converts only the uploaded ones, but it rebuilds the cell lists
    // from the staging positions, which are brought up to date first when they are not uploaded
    if (h->mixed && h->uploaded) {
        const uint64_t need = EP_MPTS_X & ~mask & ~h->fresh;
        if (need) {
            mixed_export(h->mx, h->ctx.P, h->ctx.N, h->s, false, need, false);
            CK(h, cudaGetLastError());
            h->fresh |= need;
        }
    }
    ep_mpts_view v = *m;
    for (const ViewField& f : VIEW_FIELDS)
        if (!(mask & f.bit)) v.*f.ptr = nullptr;
    return upload_view(h, &v);
}

// the control block of a fresh upload: zero, vmax from the view
static void reset_ctl(ep_handle* h, const ep_mpts_view* m) {
    std::memset(h->hctl, 0, sizeof(Ctl));
    for (int i = 0; i < h->dim; ++i) {
        double v = m->vmax ? m->vmax[i] : 0.0;
        long long bits;
        std::memcpy(&bits, &v, sizeof(double));
        h->hctl->vmax_bits[i] = (unsigned long long)bits;
    }
}

// the upload proper: every non-NULL array of the view is copied in
static ep_status upload_view(ep_handle* h, const ep_mpts_view* m) {
    HostAoS H;
    uint64_t dmask = 0;
    if (h->uploaded && direct_view(h, m, true, &H, &dmask)) {
        // one pass from the host arrays into the step's layout, binning included; the FP64 staging
        // copies of these arrays are left behind (stale until the next export)
        reset_ctl(h, m);
        CK(h, cudaMemcpyAsync(h->ctl, h->hctl, sizeof(Ctl), cudaMemcpyHostToDevice, h->s));
        mixed_import_host(h->mx, H, dmask, h->s);
        CK(h, cudaGetLastError());
        CK(h, cudaStreamSynchronize(h->s));
        h->fresh &= ~dmask;
        h->have |= dmask;
        return EP_OK;
    }
    // the copies (back to back on the copy engine), then one k_xfer over the mapped host buffers
    std::vector<XField> f = xfer_fields(h, m);
    std::vector<XField*> rest;
    XferTab T;
    int nblk = 0;
    xfer_split(f, 0, T, nblk, rest);
    for (XField* x : rest)
        CK(h, cudaMemcpyAsync(x->k > 1 ? x->stage : x->dev, x->host, x->n * sizeof(double), cudaMemcpyHostToDevice, h->s));
    if (T.n) {
        k_xfer<<<nblk, XF_BS, 0, h->s>>>(T);
        CK(h, cudaGetLastError());
    }
    // tan/sin/cos of the friction angle, evaluated on the host (material constants), again only
    // when ϕ differs from the last upload (the comparison runs while the transfers are in flight)
    const size_t np = (size_t)h->np;
    if (m->phi && (h->phi_cache.size() != np || (np && std::memcmp(h->phi_cache.data(), m->phi, np * sizeof(double)) != 0))) {
        CK(h, cudaStreamSynchronize(h->s));          // tphi_host may still be read by the last copy
        h->tphi_host.resize(3 * np);
        double* t = h->tphi_host.data();
        for (size_t p = 0; p < np; ++p) {
            t[p] = tan(m->phi[p]);
            t[np + p] = sin(m->phi[p]);
            t[2 * np + p] = cos(m->phi[p]);
        }
        h->phi_cache.assign(m->phi, m->phi + np);
        CK(h, cudaMemcpyAsync(fld_ptr(h, F_TPHI), t, 3 * np * sizeof(double), cudaMemcpyHostToDevice, h->s));
    }
    for (XField* x : rest)
        if (x->k > 1) k_aos_to_soa<<<(h->np + 255) / 256, 256, 0, h->s>>>(x->stage, x->k, h->np, x->dev);
    CK(h, cudaGetLastError());
    reset_ctl(h, m);
    CK(h, cudaMemcpyAsync(h->ctl, h->hctl, sizeof(Ctl), cudaMemcpyHostToDevice, h->s));
    // the mixed layout takes the uploaded arrays only (the others keep their device values)
    if (h->mixed) mixed_import(h->mx, h->ctx.P, h->s, view_mask(m));
    CK(h, cudaStreamSynchronize(h->s));
    CK(h, cudaGetLastError());
    h->uploaded = true;
    h->fresh |= view_mask(m);
    h->have |= view_mask(m);
    return EP_OK;
}

static ep_status read_ctl(ep_handle* h) {
    CK(h, cudaMemcpyAsync(h->hctl, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->s));
    CK(h, cudaStreamSynchronize(h->s));
    CK(h, cudaGetLastError());
    return EP_OK;
}

static ep_status kernel_error(ep_handle* h) {
    int e = h->hctl->err;
    if (!e) return EP_OK;
    char buf[160];
    if (e == EP_ERR_INVALID_POSITION)
        snprintf(buf, sizeof buf, "Invalid position: a B-spline node of point %d is outside the boundary table xB",
                 h->hctl->err_info + 1);
    else if (e == EP_ERR_NONFINITE)
        snprintf(buf, sizeof buf, "non-finite state at point %d", h->hctl->err_info + 1);
    else snprintf(buf, sizeof buf, "device error %d (info %d)", e, h->hctl->err_info);
    return fail(h, (ep_status)e, buf);
}

// one step captured once per phase: epgpu_step replays it (no per-kernel host launches); the
// eager path stays for per-kernel profiling (events between kernels)
// epgpu_step_fields's direct path as one graph: the upload of the early arrays (positions with the
// initial cell lists, v, ℓ, τ, ∇v), the step, the download of the late arrays on the stream, and two
// branches on s2 forked and joined inside the capture: the late inputs (read only by the constitutive
// pass) going up while the step's first kernels run, and x and v coming down once the G2P is done
static bool same_aos(const HostAoS& a, const HostAoS& b) { return std::memcmp(&a, &b, sizeof(HostAoS)) == 0; }
static ep_status build_fields_graph(ep_handle* h, int phase, const HostAoS& Hin, uint64_t din, const HostAoS& Hout,
                                    uint64_t dout) {
    if (h->fields_graph && h->fields_phase == phase && h->fields_in == din && h->fields_out == dout &&
        same_aos(h->fields_hin, Hin) && same_aos(h->fields_hout, Hout))
        return EP_OK;
    if (h->fields_graph) cudaGraphExecDestroy(h->fields_graph);
    h->fields_graph = nullptr;
    h->fields_phase = -1;
    constexpr uint64_t LATE_IN = EP_MPTS_FIJ | EP_MPTS_BIJ | EP_MPTS_EPII | EP_MPTS_DLAM;
    constexpr uint64_t EARLY_OUT = EP_MPTS_X | EP_MPTS_V;
    const uint64_t late_in = din & LATE_IN, early_out = dout & EARLY_OUT;
    cudaGraph_t gr;
    const long long l0 = h->launches;
    CK(h, cudaStreamBeginCapture(h->s, cudaStreamCaptureModeThreadLocal));
    mixed_import_host(h->mx, Hin, din & ~late_in, h->s);
    if (late_in) {
        cudaEventRecord(h->ev_up, h->s);                           // one link direction: in turn
        cudaStreamWaitEvent(h->s2, h->ev_up, 0);
        mixed_import_host(h->mx, Hin, late_in, h->s2, false);
        cudaEventRecord(h->ev_late, h->s2);
    }
    cudaEventRecordWithFlags(h->ev0, h->s, cudaEventRecordExternal);
    MixedCtx mx = h->mx;
    mx.begin_step = 1;
    mx.hooks_internal = true;
    mx.ev_need = late_in ? h->ev_late : nullptr;                  // joined before the constitutive pass
    mx.ev_moved = early_out ? h->ev_moved : nullptr;              // forked after the G2P
    mixed_step(mx, phase, h->s);
    cudaEventRecordWithFlags(h->ev1, h->s, cudaEventRecordExternal);
    if (early_out) {
        // reset_ctl starts the step at parity 0: its G2P writes the offsets of parity 1
        cudaStreamWaitEvent(h->s2, h->ev_moved, 0);
        mixed_export_host(h->mx, Hout, early_out, h->s2, 1);
        cudaEventRecord(h->ev_dn, h->s2);
    }
    mixed_export_host(h->mx, Hout, dout & ~early_out, h->s);
    if (early_out) cudaStreamWaitEvent(h->s, h->ev_dn, 0);
    cudaError_t e = cudaStreamEndCapture(h->s, &gr);
    h->fields_kernels = h->launches - l0;
    h->launches = l0;
    if (e != cudaSuccess) return cuda_fail(h, e, "step_fields graph capture");
    e = cudaGraphInstantiate(&h->fields_graph, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) return cuda_fail(h, e, "step_fields graph instantiate");
    h->fields_phase = phase;
    h->fields_in = din;
    h->fields_out = dout;
    h->fields_hin = Hin;
    h->fields_hout = Hout;
    return EP_OK;
}

static ep_status build_step_graph(ep_handle* h, int phase) {
    if (h->step_graph[phase]) return EP_OK;
    cudaGraph_t gr;
    long long l0 = h->launches;
    CK(h, cudaStreamBeginCapture(h->s, cudaStreamCaptureModeThreadLocal));
    if (h->mixed) {
        // the mixed step's first kernel (km_zero) starts the step itself
        MixedCtx mx = h->mx;
        mx.begin_step = 1;
        mixed_step(mx, phase, h->s);
    } else {
        launch_ctl_begin_step(h->ctl, h->dim, h->s);
        fp64_step(h->ctx, phase, h->s);
        h->launches += 1;                              // the control kernel
    }
    cudaError_t e = cudaStreamEndCapture(h->s, &gr);
    h->step_kernels[phase] = h->launches - l0;
    h->launches = l0;
    if (e != cudaSuccess) return cuda_fail(h, e, "step graph capture");
    e = cudaGraphInstantiate(&h->step_graph[phase], gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) return cuda_fail(h, e, "step graph instantiate");
    return EP_OK;
}

ep_status epgpu_step(ep_handle* h, int32_t phase, double dt, const double* g, double* vmax_out) {
    if (!h || !g) return EP_ERR_ARG;
    if (!h->uploaded) return fail(h, EP_ERR_STATE, "step before upload");
    if (phase != 0 && phase != 1) return fail(h, EP_ERR_ARG, "phase must be 0 or 1");
    ep_status st;
    if (!h->prof.on && (st = build_step_graph(h, phase)) != EP_OK) return st;
    // the step's dt, g and phase into the device control block by a one-thread kernel (no host round
    // trip: the block's other fields are the device's own, read back after the step)
    double gg[3];
    for (int i = 0; i < 3; ++i) gg[i] = i < h->dim ? g[i] : 0.0;
    launch_ctl_set_step(h->ctl, dt, gg, phase, h->s);
    CK(h, cudaGetLastError());
    CK(h, cudaEventRecord(h->ev0, h->s));
    if (!h->prof.on) {
        CK(h, cudaGraphLaunch(h->step_graph[phase], h->s));
        h->launches += h->step_kernels[phase];
    } else {
        // the step as the timed graph runs it, captured with an event recorded after every kernel:
        // the per-kernel times hold no host launch gaps
        if (h->prof_phase != phase) {
            if (h->prof_graph) cudaGraphExecDestroy(h->prof_graph);
            h->prof_graph = nullptr;
            h->prof_phase = -1;
            const long long l0 = h->launches;
            h->prof.reserve(64);
            cudaGraph_t gr;
            CK(h, cudaStreamBeginCapture(h->s, cudaStreamCaptureModeThreadLocal));
            Fp64Ctx ctx = h->ctx;
            ctx.prof = &h->prof;
            if (!h->mixed) {
                launch_ctl_begin_step(h->ctl, h->dim, h->s);
                h->launches += 1;
            }
            h->prof.begin(h->s);
            if (h->mixed) {
                MixedCtx mx = h->mx;
                mx.prof = &h->prof;
                mx.begin_step = 1;
                mixed_step(mx, phase, h->s);
            } else {
                fp64_step(ctx, phase, h->s);
            }
            cudaError_t e = cudaStreamEndCapture(h->s, &gr);
            h->prof_kernels = h->launches - l0;
            h->launches = l0;
            if (e != cudaSuccess) return cuda_fail(h, e, "profiled step capture");
            e = cudaGraphInstantiate(&h->prof_graph, gr, 0);
            cudaGraphDestroy(gr);
            if (e != cudaSuccess) return cuda_fail(h, e, "profiled step instantiate");
            h->prof_phase = phase;
            h->prof_n = h->prof.n;
            h->prof_names.assign(h->prof.name.begin(), h->prof.name.begin() + h->prof.n);
        }
        h->prof.n = h->prof_n;
        for (int i = 0; i < h->prof_n; ++i) h->prof.name[i] = h->prof_names[i];
        CK(h, cudaGraphLaunch(h->prof_graph, h->s));
        h->launches += h->prof_kernels;
    }
    CK(h, cudaEventRecord(h->ev1, h->s));
    CK(h, cudaGetLastError());
    if ((st = read_ctl(h)) != EP_OK) return st;
    h->prof.collect();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    h->last_ms = ms;
    h->steps += 1;
    h->fresh = 0;
    if (vmax_out)
        for (int i = 0; i < h->dim; ++i) vmax_out[i] = bits_to_double(h->hctl->vmax_bits[i]);
    return kernel_error(h);
}

static ep_status build_graph(ep_handle* h, int phase) {
    if (h->graph[phase]) return EP_OK;
    cudaGraph_t gr;
    long long l0 = h->launches;
    CK(h, cudaStreamBeginCapture(h->s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < GRAPH_STEPS; ++k) {
        launch_ctl_begin_run(h->ctl, h->ctx.g, h->cm.c, h->s);
        if (h->mixed) mixed_step(h->mx, phase, h->s);
        else fp64_step(h->ctx, phase, h->s);
        launch_ctl_end(h->ctl, h->s);
    }
    cudaError_t e = cudaStreamEndCapture(h->s, &gr);
    h->graph_kernels[phase] = h->launches - l0 + 2LL * GRAPH_STEPS;   // + control kernels
    h->launches = l0;                                                    // capturing launches nothing
    if (e != cudaSuccess) return cuda_fail(h, e, "graph capture");
    e = cudaGraphInstantiate(&h->graph[phase], gr, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(gr);
        return cuda_fail(h, e, "graph instantiate");
    }
    h->graph_def[phase] = gr;
    return EP_OK;
}

ep_status epgpu_run(ep_handle* h, int32_t phase, double T, double tg, double* t_inout, int64_t* nsteps_out) {
    if (!h || !t_inout) return EP_ERR_ARG;
    if (!h->uploaded) return fail(h, EP_ERR_STATE, "run before upload");
    if (phase != 0 && phase != 1) return fail(h, EP_ERR_ARG, "phase must be 0 or 1");
    ep_status st;
    if ((st = read_ctl(h)) != EP_OK) return st;
    if (h->hctl->err) return kernel_error(h);
    h->hctl->t = *t_inout;
    h->hctl->T = T;
    h->hctl->tg = tg;
    h->hctl->phase = phase;
    h->hctl->active = 1;
    h->hctl->nsteps = 0;
    CK(h, cudaMemcpyAsync(h->ctl, h->hctl, sizeof(Ctl), cudaMemcpyHostToDevice, h->s));
    if ((st = build_graph(h, phase)) != EP_OK) return st;
    CK(h, cudaEventRecord(h->ev0, h->s));
    int launched = 0;
    while (true) {
        CK(h, cudaGraphLaunch(h->graph[phase], h->s));
        ++launched;
        if ((st = read_ctl(h)) != EP_OK) return st;
        if (!h->hctl->active || h->hctl->err) break;
        if (launched >= (1 << 24)) return fail(h, EP_ERR_TIMEOUT, "time loop did not reach T after 2^28 steps");
    }
    CK(h, cudaEventRecord(h->ev1, h->s));
    CK(h, cudaEventSynchronize(h->ev1));
    h->launches += launched * h->graph_kernels[phase];
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    h->last_ms = ms;
    *t_inout = h->hctl->t;
    h->t = h->hctl->t;
    h->steps += h->hctl->nsteps;
    h->fresh = 0;
    if (nsteps_out) *nsteps_out = h->hctl->nsteps;
    return kernel_error(h);
}

ep_status epgpu_run_checkpoints(ep_handle* h, int32_t phase, const double* checkpoints, int32_t ncheck,
                                double tg, double* t_inout, ep_checkpoint_cb cb, void* user, int64_t* nsteps_out) {
    if (!h || !t_inout || ncheck < 0 || (ncheck > 0 && !checkpoints)) return EP_ERR_ARG;
    std::vector<double> checks(checkpoints, checkpoints + ncheck);
    for (double T : checks)
        if (!std::isfinite(T)) return fail(h, EP_ERR_ARG, "a checkpoint time is not finite");
    std::sort(checks.begin(), checks.end());
    int64_t total = 0;
    for (int32_t k = 0; k < ncheck; ++k) {
        int64_t n = 0;
        ep_status st = epgpu_run(h, phase, checks[k], tg, t_inout, &n);
        total += n;
        if (nsteps_out) *nsteps_out = total;
        if (st != EP_OK) return st;
        if (cb && cb(h, k, *t_inout, user) != 0) break;
    }
    if (nsteps_out) *nsteps_out = total;
    return EP_OK;
}

static ep_status download_view(ep_handle* h, ep_mpts_view* m, bool need_eps);

// the view restricted to the arrays of `mask` (topology left out)
static ep_mpts_view masked_view(const ep_mpts_view* m, uint64_t mask) {
    ep_mpts_view v = *m;
    for (const ViewField& f : VIEW_FIELDS)
        if (!(mask & f.bit)) v.*f.ptr = nullptr;
    v.p2e = nullptr;
    v.p2n = nullptr;
    return v;
}

ep_status epgpu_step_fields(ep_handle* h, ep_mpts_view* m, uint64_t mask_in, int32_t phase, double dt,
                            const double* g, uint64_t mask_out, double* vmax_out) {
    if (!h || !m || !g) return EP_ERR_ARG;
    if (m->nmp != h->np || m->ndim != h->dim) return fail(h, EP_ERR_ARG, "mpts.nmp/ndim differ from create");
    if ((mask_in | mask_out) & ~EP_MPTS_ALL) return fail(h, EP_ERR_ARG, "unknown bits in the field mask");
    if (phase != 0 && phase != 1) return fail(h, EP_ERR_ARG, "phase must be 0 or 1");
    const uint64_t given = view_mask(m);
    if ((mask_in | mask_out) & ~given)
        return fail(h, EP_ERR_ARG, "a field in the mask is NULL: " + mask_names((mask_in | mask_out) & ~given));
    ep_mpts_view vin = masked_view(m, mask_in), vout = masked_view(m, mask_out);
    HostAoS Hin, Hout;
    uint64_t din = 0, dout = 0;
    const bool direct = h->uploaded && !h->prof.on && !(reads_of(h) & ~(mask_in | h->have)) &&
                        direct_view(h, &vin, true, &Hin, &din) && direct_view(h, &vout, false, &Hout, &dout);
    if (!direct) {
        ep_status st = epgpu_upload_fields(h, m, mask_in);
        if (st == EP_OK) st = epgpu_step(h, phase, dt, g, vmax_out);
        if (st == EP_OK) st = epgpu_download_fields(h, m, mask_out);
        return st;
    }
    // upload (as upload_view's direct path), the step (as epgpu_step) and the download (as
    // download_view's direct path) queued on the device with one synchronisation.  The link's two
    // directions and the step overlap: the arrays only the constitutive pass reads (F, b_e, ϵpII, Δλ)
    // follow the rest of the upload on a second stream while the step's first kernels run, and the
    // positions and velocities, final after the G2P, go down on that stream during the rest of the step.
    if (!h->s2) {
        cudaError_t e = cudaStreamCreateWithFlags(&h->s2, cudaStreamNonBlocking);
        for (cudaEvent_t* ev : {&h->ev_up, &h->ev_late, &h->ev_moved, &h->ev_dn})
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(h, e, "step_fields: second stream");
    }
    ep_status st;
    if ((st = build_fields_graph(h, phase, Hin, din, Hout, dout)) != EP_OK) return st;
    reset_ctl(h, &vin);
    CK(h, cudaMemcpyAsync(h->ctl, h->hctl, sizeof(Ctl), cudaMemcpyHostToDevice, h->s));
    double gg[3];
    for (int i = 0; i < 3; ++i) gg[i] = i < h->dim ? g[i] : 0.0;
    launch_ctl_set_step(h->ctl, dt, gg, phase, h->s);
    CK(h, cudaGetLastError());
    CK(h, cudaGraphLaunch(h->fields_graph, h->s));                // ev0 and ev1 bracket the step inside
    h->launches += h->fields_kernels;
    CK(h, cudaGetLastError());
    if ((st = read_ctl(h)) != EP_OK) return st;              // synchronizes: the host arrays are written
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    h->last_ms = ms;
    h->steps += 1;
    h->have |= din;
    h->fresh = 0;
    for (int i = 0; i < h->dim; ++i) {
        const double v = bits_to_double(h->hctl->vmax_bits[i]);
        if (vmax_out) vmax_out[i] = v;
        if (m->vmax) m->vmax[i] = v;                          // as epgpu_download_fields
    }
    return kernel_error(h);
}

ep_status epgpu_download(ep_handle* h, ep_mpts_view* m) {
    if (!h || !m) return EP_ERR_ARG;
    if (m->nmp != h->np || m->ndim != h->dim) return fail(h, EP_ERR_ARG, "mpts.nmp/ndim differ from create");
    return download_view(h, m, true);
}

ep_status epgpu_download_fields(ep_handle* h, ep_mpts_view* m, uint64_t mask) {
    if (!h || !m) return EP_ERR_ARG;
    if (m->nmp != h->np || m->ndim != h->dim) return fail(h, EP_ERR_ARG, "mpts.nmp/ndim differ from create");
    if (mask & ~EP_MPTS_ALL) return fail(h, EP_ERR_ARG, "unknown bits in the field mask");
    const uint64_t given = view_mask(m);
    if (mask & ~given) return fail(h, EP_ERR_ARG, "a field in the mask is NULL: " + mask_names(mask & ~given));
    ep_mpts_view v = *m;
    for (const ViewField& f : VIEW_FIELDS)
        if (!(mask & f.bit)) v.*f.ptr = nullptr;
    v.p2e = nullptr;
    v.p2n = nullptr;
    return download_view(h, &v, (mask & EP_MPTS_EIJ) != 0);
}

static ep_status download_view(ep_handle* h, ep_mpts_view* m, bool need_eps) {
    const int d = h->dim;
    ep_status st;
    HostAoS H;
    uint64_t dmask = 0;
    if (h->uploaded && direct_view(h, m, false, &H, &dmask)) {
        // one pass from the step's layout into the host arrays (no FP64 staging)
        mixed_export_host(h->mx, H, dmask, h->s);
        CK(h, cudaGetLastError());
        if ((st = read_ctl(h)) != EP_OK) return st;      // synchronizes: the host arrays are written
        if (m->vmax)
            for (int i = 0; i < d; ++i) m->vmax[i] = bits_to_double(h->hctl->vmax_bits[i]);
        return EP_OK;
    }
    if (h->mixed && h->uploaded) {
        // the requested point arrays only (the nodal fields are download_mesh's)
        const uint64_t want = view_mask(m);
        mixed_export(h->mx, h->ctx.P, h->ctx.N, h->s, need_eps, want, false);
        CK(h, cudaGetLastError());
        h->fresh |= want;
    }
    if ((st = read_ctl(h)) != EP_OK) return st;
    // one k_xfer into the mapped host buffers; the other fields transposed into staging, then
    // copied back to back
    std::vector<XField> f = xfer_fields(h, m);
    std::vector<XField*> rest;
    XferTab T;
    int nblk = 0;
    xfer_split(f, 1, T, nblk, rest);
    if (T.n) k_xfer<<<nblk, XF_BS, 0, h->s>>>(T);
    for (XField* x : rest)
        if (x->k > 1) k_soa_to_aos<<<(h->np + 255) / 256, 256, 0, h->s>>>(x->dev, x->k, h->np, x->stage);
    CK(h, cudaGetLastError());
    for (XField* x : rest)
        CK(h, cudaMemcpyAsync(x->host, x->k > 1 ? x->stage : x->dev, x->n * sizeof(double), cudaMemcpyDeviceToHost, h->s));
    if (m->vmax)
        for (int i = 0; i < d; ++i) m->vmax[i] = bits_to_double(h->hctl->vmax_bits[i]);
    CK(h, cudaStreamSynchronize(h->s));
    if (m->p2e || m->p2n) {
        std::vector<int> c(h->np);
        if (h->np) {
            CK(h, cudaMemcpyAsync(c.data(), h->ctx.P.p2e, sizeof(int) * h->np, cudaMemcpyDeviceToHost, h->s));
            CK(h, cudaStreamSynchronize(h->s));
        }
        for (int p = 0; p < h->np; ++p) {
            if (m->p2e) m->p2e[p] = (int64_t)c[p] + 1;
            if (!m->p2n) continue;
            int e[3];
            if (d == 2) { e[0] = c[p] / (int)h->nel[1]; e[1] = c[p] % (int)h->nel[1]; }
            else {
                int nzx = (int)(h->nel[2] * h->nel[0]);
                e[1] = c[p] / nzx;
                int r = c[p] % nzx;
                e[0] = r / (int)h->nel[2];
                e[2] = r % (int)h->nel[2];
            }
            for (int s = 0; s < h->nn; ++s) {
                int o[3], i[3];
                if (d == 2) { o[0] = s >> 2; o[1] = s & 3; }
                else { o[1] = s >> 4; o[0] = (s >> 2) & 3; o[2] = s & 3; }
                bool ok = c[p] >= 0;
                for (int dd = 0; dd < d; ++dd) {
                    i[dd] = e[dd] - 1 + o[dd];
                    ok = ok && i[dd] >= 0 && i[dd] < h->nno[dd];
                }
                long long id = 0;
                if (ok) id = (d == 2) ? i[1] + h->nno[1] * (long long)i[0]
                                      : i[2] + h->nno[2] * (long long)i[0] + h->nno[2] * h->nno[0] * (long long)i[1];
                m->p2n[s + (int64_t)h->nn * p] = ok ? id + 1 : 0;
            }
        }
    }
    return EP_OK;
}

// savlot's plot fields (plot.jl:27-135) from the FP64 SoA state, one row of np per requested field in
// bit order; products and sums rounded one by one as plot.jl's broadcasts do (no contraction)
struct FieldSrc {
    const double *s0, *s1, *s2, *eps, *ep, *u, *epv, *c0, *n, *J, *rho, *om, *x, *z;
    int dim;
};

__global__ void k_fields(const FieldSrc S, uint32_t what, int np, double* out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    int row = 0;
    auto put = [&](double v) { out[(size_t)row++ * np + p] = v; };
    if (what & EP_FIELD_P) {
        if (S.dim == 2) put(-__dadd_rn(S.s0[p], S.s1[p]) / 2.0 / 1e3);
        else put(-__dadd_rn(__dadd_rn(S.s0[p], S.s1[p]), S.s2[p]) / 3.0 / 1e3);
    }
    if (what & EP_FIELD_SIGXX) put(S.s0[p] / 1e3);
    if (what & EP_FIELD_EPSXX) put(S.eps[p]);
    if (what & EP_FIELD_EPII) put(S.ep[p]);
    if (what & EP_FIELD_EPV) put(S.epv[p]);
    if (what & EP_FIELD_DU) {
        const double a = S.u[(size_t)S.dim * p], b = S.u[(size_t)S.dim * p + 1];
        put(sqrt(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b))));
    }
    if (what & EP_FIELD_COH0) put(S.c0[p] / 1e3);
    if (what & EP_FIELD_PHI0) ++row;   // ϕ is not held on the device: the host fills this row
    if (what & EP_FIELD_N) put(S.n[p]);
    if (what & EP_FIELD_J) put(S.J[p]);
    if (what & EP_FIELD_MS) put(__dmul_rn(S.rho[p], S.om[p]));
    if (what & EP_FIELD_X) put(S.x[p]);
    if (what & EP_FIELD_Z) put(S.z[p]);
}

ep_status epgpu_fields(ep_handle* h, uint32_t what, double* out) {
    if (!h) return EP_ERR_ARG;
    if (what & ~EP_FIELD_ALL) return fail(h, EP_ERR_ARG, "UndefinedPlotOption: unknown bits in the field mask");
    if (what && !out) return fail(h, EP_ERR_ARG, "fields: out is NULL");
    if (!h->uploaded) return fail(h, EP_ERR_STATE, "fields before upload");
    const size_t np = (size_t)h->np;
    if (!what || np == 0) return EP_OK;
    const int d = h->dim;
    if (h->mixed) {
        mixed_export(h->mx, h->ctx.P, h->ctx.N, h->s);
        CK(h, cudaGetLastError());
        h->fresh = EP_MPTS_ALL;
    }
    FieldSrc S;
    const double* sig = fld_ptr(h, F_SIG);
    S.s0 = sig;
    S.s1 = sig + np;
    S.s2 = sig + 2 * np;
    S.eps = fld_ptr(h, F_EPS);
    S.ep = fld_ptr(h, F_EP);
    S.u = h->pass;
    S.epv = h->pass + (2 + (size_t)d) * d * np;
    S.c0 = fld_ptr(h, F_C0);
    S.n = fld_ptr(h, F_N);
    S.J = fld_ptr(h, F_J);
    S.rho = fld_ptr(h, F_RHO);
    S.om = fld_ptr(h, F_OM);
    S.x = fld_ptr(h, F_X);
    S.z = fld_ptr(h, F_X) + (size_t)(d - 1) * np;
    S.dim = d;
    const int rows = __builtin_popcount(what);
    k_fields<<<(unsigned)((np + 255) / 256), 256, 0, h->s>>>(S, what, (int)np, h->xfer);   // staging: >= 13 rows
    CK(h, cudaGetLastError());
    CK(h, cudaMemcpyAsync(out, h->xfer, (size_t)rows * np * sizeof(double), cudaMemcpyDeviceToHost, h->s));
    CK(h, cudaStreamSynchronize(h->s));
    if (what & EP_FIELD_PHI0) {
        const int row = __builtin_popcount(what & (EP_FIELD_PHI0 - 1u));
        std::memcpy(out + (size_t)row * np, h->phi_cache.data(), np * sizeof(double));
    }
    return EP_OK;
}

ep_status epgpu_download_mesh(ep_handle* h, ep_mesh_fields* f) {
    if (!h || !f) return EP_ERR_ARG;
    const int d = h->dim;
    const size_t Nn = h->nnode;
    if (h->mixed && h->uploaded) {
        mixed_export(h->mx, h->ctx.P, h->ctx.N, h->s, false);
        CK(h, cudaGetLastError());
        h->fresh = EP_MPTS_ALL;
    }
    std::vector<double> buf((size_t)(1 + 4 * d + 1) * Nn);
    CK(h, cudaMemcpyAsync(buf.data(), h->nbuf, buf.size() * sizeof(double), cudaMemcpyDeviceToHost, h->s));
    CK(h, cudaStreamSynchronize(h->s));
    auto aos = [&](size_t base, double* out) {
        if (!out) return;
        for (size_t n = 0; n < Nn; ++n)
            for (int i = 0; i < d; ++i) out[i + d * n] = buf[base + i * Nn + n];
    };
    if (f->mi) std::memcpy(f->mi, buf.data(), Nn * sizeof(double));
    aos(1 * Nn, f->p);
    aos((1 + d) * Nn, f->oobf);
    aos((1 + 2 * (size_t)d) * Nn, f->a);
    aos((1 + 3 * (size_t)d) * Nn, f->v);
    if (f->dJ) std::memcpy(f->dJ, buf.data() + (1 + 4 * (size_t)d) * Nn, Nn * sizeof(double));
    return EP_OK;
}

ep_status epgpu_profile(ep_handle* h, int32_t enable) {
    if (!h) return EP_ERR_ARG;
    h->prof.on = enable != 0;
    if (enable) h->prof.acc.clear();
    return EP_OK;
}

ep_status epgpu_profile_read(ep_handle* h, ep_kernel_time* out, int32_t cap, int32_t* count) {
    if (!h || !count || (cap > 0 && !out)) return EP_ERR_ARG;
    int i = 0;
    for (auto& kv : h->prof.acc) {
        if (i < cap) {
            std::memset(out[i].name, 0, sizeof(out[i].name));
            std::strncpy(out[i].name, kv.first.c_str(), sizeof(out[i].name) - 1);
            out[i].launches = kv.second.first;
            out[i].total_ms = kv.second.second;
        }
        ++i;
    }
    *count = i;
    return EP_OK;
}

ep_status epgpu_stats(ep_handle* h, ep_stats* out) {
    if (!h || !out) return EP_ERR_ARG;
    ep_status st;
    if ((st = read_ctl(h)) != EP_OK) return st;
    out->steps = h->steps;
    out->launches = h->launches;
    out->device_ms = h->last_ms;
    out->t = h->t;
    out->plastic = h->hctl->plastic;
    return EP_OK;
}

// ---------------------------------------------------------------------------
// Conservation sums in FP64 (epgpu_conservation).  Fixed-order reductions: block b sums the points (or
// nodes) [b*chunk, (b+1)*chunk) with thread t taking every 256th one from b*chunk + t in ascending order,
// then a shared-memory tree in a fixed pairing; one block then adds the SUM_BLOCKS partials the same
// way.  The result depends only on the data, not on scheduling.
// Quantities: 0 Σ ρΩ, 1-3 Σ ρΩ v, 4 ½ Σ ρΩ |v|², 5 ½ Σ Ω τ·Del⁻¹τ, 6 Σ m_n, 7-9 Σ p_n.
struct SumSrc {
    const double *rho, *om, *om0, *v[3], *st[6];
    const double *m, *p[3];
    int np, nnode, dim, ns, fin;
};

__device__ __forceinline__ double elastic_energy(const Mat& mt, const double* st, int ns) {
    double x[6];
    if (ns == 3) lu_solve<3>(mt.DelLU, mt.piv, st, x);
    else lu_solve<6>(mt.DelLU, mt.piv, st, x);
    double w = st[0] * x[0];
    for (int i = 1; i < ns; ++i) w = w + st[i] * x[i];
    return 0.5 * w;
}

__device__ __forceinline__ void block_sum_fixed(double* sh, double* q, int nq, double* out) {
    const int t = threadIdx.x;
    for (int k = 0; k < nq; ++k) sh[k * 256 + t] = q[k];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w)
            for (int k = 0; k < nq; ++k) sh[k * 256 + t] = sh[k * 256 + t] + sh[k * 256 + t + w];
        __syncthreads();
    }
    if (t < nq) out[t] = sh[t * 256];
}

__global__ void __launch_bounds__(256) k_sums(const SumSrc S, const Mat mt, double* part) {
    __shared__ double sh[SUM_Q * 256];
    double q[SUM_Q];
    for (int k = 0; k < SUM_Q; ++k) q[k] = 0.0;
    const int b = blockIdx.x, t = threadIdx.x;
    const int pc = (S.np + SUM_BLOCKS - 1) / SUM_BLOCKS, nc = (S.nnode + SUM_BLOCKS - 1) / SUM_BLOCKS;
    const int p0 = b * pc, p1 = min(S.np, p0 + pc);
    for (int p = p0 + t; p < p1; p += 256) {
        const double m = S.rho[p] * S.om[p];
        double v2 = 0.0;
        q[0] = q[0] + m;
        for (int d = 0; d < S.dim; ++d) {
            const double v = S.v[d][p];
            q[1 + d] = q[1 + d] + m * v;
            v2 = v2 + v * v;
        }
        q[4] = q[4] + 0.5 * (m * v2);
        double st[6];
        for (int k = 0; k < S.ns; ++k) st[k] = S.st[k][p];
        const double w = elastic_energy(mt, st, S.ns);
        q[5] = q[5] + w * (S.fin ? S.om0[p] : S.om[p]);
    }
    const int n0 = b * nc, n1 = min(S.nnode, n0 + nc);
    for (int n = n0 + t; n < n1; n += 256) {
        q[6] = q[6] + S.m[n];
        for (int d = 0; d < S.dim; ++d) q[7 + d] = q[7 + d] + S.p[d][n];
    }
    block_sum_fixed(sh, q, SUM_Q, part + (size_t)b * SUM_Q);
}

__global__ void __launch_bounds__(256) k_sums_final(const double* part, double* out) {
    __shared__ double sh[SUM_Q * 256];
    double q[SUM_Q];
    for (int k = 0; k < SUM_Q; ++k) q[k] = 0.0;
    for (int b = threadIdx.x; b < SUM_BLOCKS; b += 256)
        for (int k = 0; k < SUM_Q; ++k) q[k] = q[k] + part[(size_t)b * SUM_Q + k];
    block_sum_fixed(sh, q, SUM_Q, out);
}

ep_status epgpu_conservation(ep_handle* h, ep_conservation* out) {
    if (!h || !out) return EP_ERR_ARG;
    if (!h->uploaded) return fail(h, EP_ERR_STATE, "conservation sums before upload");
    const int d = h->dim;
    if (h->mixed) {
        mixed_export(h->mx, h->ctx.P, h->ctx.N, h->s, false);
        CK(h, cudaGetLastError());
        h->fresh = EP_MPTS_ALL;
    }
    const P64& P = h->ctx.P;
    const N64& N = h->ctx.N;
    SumSrc S{};
    S.rho = P.rho;
    S.om = P.Om;
    S.om0 = P.Om0;
    S.fin = h->cfg.deform == EP_DEFORM_FINITE;
    for (int i = 0; i < d; ++i) {
        S.v[i] = P.v[i];
        S.p[i] = N.p[i];
    }
    S.ns = h->nstr;
    for (int k = 0; k < h->nstr; ++k) S.st[k] = S.fin ? P.tau[k] : P.sig[k];
    S.m = N.m;
    S.np = h->np;
    S.nnode = h->nnode;
    S.dim = d;
    k_sums<<<SUM_BLOCKS, 256, 0, h->s>>>(S, h->ctx.mt, h->sums);
    k_sums_final<<<1, 256, 0, h->s>>>(h->sums, h->sums + (size_t)SUM_BLOCKS * SUM_Q);
    CK(h, cudaGetLastError());
    double q[SUM_Q];
    CK(h, cudaMemcpyAsync(q, h->sums + (size_t)SUM_BLOCKS * SUM_Q, sizeof q, cudaMemcpyDeviceToHost, h->s));
    CK(h, cudaStreamSynchronize(h->s));
    std::memset(out, 0, sizeof *out);
    out->mass = q[0];
    out->kinetic = q[4];
    out->elastic = q[5];
    out->mass_nodes = q[6];
    for (int i = 0; i < d; ++i) {
        out->momentum[i] = q[1 + i];
        out->momentum_nodes[i] = q[7 + i];
    }
    return EP_OK;
}

ep_status epgpu_set_return_map(ep_handle* h, ep_mlp* m, int32_t mode) {
    if (!h) return EP_ERR_ARG;
    if (mode != EP_RMAP_EXACT && mode != EP_RMAP_LEARNED && mode != EP_RMAP_RECORD)
        return fail(h, EP_ERR_ARG, "return map mode must be EP_RMAP_EXACT, _LEARNED or _RECORD");
    if (mode != EP_RMAP_EXACT) {
        if (!m) return fail(h, EP_ERR_ARG, "a network is required for the learned and record modes");
        if (!h->mixed || h->cfg.deform != EP_DEFORM_FINITE || h->cfg.constitutive != EP_CONS_DP)
            return fail(h, EP_ERR_UNSUPPORTED,
                        "the learned return map stands in for the finite-strain DP return of the mixed step");
        if (mode == EP_RMAP_RECORD && mlp_record_cap(m) <= 0)
            return fail(h, EP_ERR_STATE, "the network has no record buffer (epgpu_mlp_record_buffer)");
    }
    RmapBufs b{};
    b.mode = mode;
    if (mode == EP_RMAP_LEARNED) {
        const size_t np = (size_t)std::max(h->np, 1);
        const size_t naux = h->dim == 2 ? 4 : 12;    // per slot: (cos 2θ, sin 2θ, s, c) or (V, s, c, 0)
        if (!h->rm_buf) {
            if (dalloc(h, &h->rm_buf, np * (RM_NX + RM_NY + naux)) != cudaSuccess ||
                dalloc(h, &h->rm_int, 2 * np + 2) != cudaSuccess)
                return fail(h, EP_ERR_NOMEM, "device allocation (learned return map slots)");
        }
        b.rx = h->rm_buf;
        b.ry = h->rm_buf + np * RM_NX;
        b.raux = h->rm_buf + np * (RM_NX + RM_NY);
        b.rcount = h->rm_int;
        b.fbcount = h->rm_int + 1;
        b.rpt = h->rm_int + 2;
        b.fblist = h->rm_int + 2 + np;
        CK(h, cudaMemsetAsync(b.rcount, 0, 2 * sizeof(int), h->s));
    } else if (mode == EP_RMAP_RECORD) {
        b.rx = mlp_record_x(m);
        b.ry = mlp_record_t(m);
        b.rec_count = mlp_record_count(m);
        b.rec_cap = mlp_record_cap(m);
    }
    if (h->mixed) {
        mixed_set_rmap(h->mx_impl.data(), b);
        h->mx.net = mode == EP_RMAP_LEARNED ? m : nullptr;
        drop_graphs(h);                               // the captured kernels hold the old argument block
    }
    h->rm_net = m;
    h->rm_mode = mode;
    ep_status st;
    if ((st = read_ctl(h)) != EP_OK) return st;
    h->hctl->rm_learned = 0;
    h->hctl->rm_fallback = 0;
    CK(h, cudaMemcpyAsync(h->ctl, h->hctl, sizeof(Ctl), cudaMemcpyHostToDevice, h->s));
    CK(h, cudaStreamSynchronize(h->s));
    return EP_OK;
}

ep_status epgpu_return_map_stats(ep_handle* h, int64_t* learned, int64_t* fallback, int64_t* recorded) {
    if (!h) return EP_ERR_ARG;
    ep_status st;
    if ((st = read_ctl(h)) != EP_OK) return st;
    if (learned) *learned = (int64_t)h->hctl->rm_learned;
    if (fallback) *fallback = (int64_t)h->hctl->rm_fallback;
    if (recorded) {
        long long c = 0;
        if (h->rm_mode == EP_RMAP_RECORD && h->rm_net) {
            CK(h, cudaMemcpyAsync(&c, mlp_record_count(h->rm_net), sizeof(long long), cudaMemcpyDeviceToHost, h->s));
            CK(h, cudaStreamSynchronize(h->s));
        }
        *recorded = c;
    }
    return EP_OK;
}

// ---------------------------------------------------------------------------
// Batched ensemble (no counterpart in the reference, which runs one slump per
// process): independent instances, each with its own mesh, points, switches and
// time loop, advanced together.  Every instance keeps its own device state and
// 16-step graph; the batch graph holds those graphs as child nodes with no
// dependencies between them, so one launch advances every instance by up to 16
// of its own steps (instances past their window return at once), followed by one
// kernel that gathers the instances' active / error words.
__global__ void k_batch_flags(Ctl* const* ctls, int n, int* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = (ctls[i]->active ? 1 : 0) | (ctls[i]->err ? 2 : 0);
}

struct ep_batch {
    std::vector<ep_handle*> h;
    cudaStream_t s = nullptr;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    Ctl** dctl = nullptr;         // device array of the instances' control blocks
    int* dflags = nullptr;
    int* hflags = nullptr;        // pinned
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0.0;
    long long launches = 0;
    std::string err;
    // one persistent kernel for all instances (2d mixed, exact map), else per-instance graphs
    void* pimpl = nullptr;
    bool ptried = false;
    std::string pwhy;
    int tile = 64;
    // -1 default (phase kernels when the batch qualifies), 0 instance graphs, 1 persistent kernel,
    // 2 phase kernels over all instances
    int scheme = -1;
    double tune_ms[9] = {};       // autotuner: schemes 0, 1, 2 x tiles 16 / 32 / 64
    int used_scheme() const { return pimpl ? (scheme < 0 ? 2 : scheme) : 0; }
    std::vector<int> gens;        // the instances' graph generations the batch graphs were built from
};

static ep_status bfail(ep_batch* b, ep_status st, const std::string& m) {
    if (b) b->err = m;
    else g_create_error = m;
    return st;
}
#define BCK(b, call)                                                                   \
    do {                                                                               \
        cudaError_t e__ = (call);                                                      \
        if (e__ != cudaSuccess) {                                                      \
            cudaGetLastError();                                                        \
            return bfail((b), EP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e__)); \
        }                                                                              \
    } while (0)

static void batch_drop(ep_batch* b) {
    for (int k = 0; k < 2; ++k)
        if (b->exec[k]) {
            cudaGraphExecDestroy(b->exec[k]);
            b->exec[k] = nullptr;
        }
    if (b->pimpl) mixed_batch_destroy(b->pimpl);
    b->pimpl = nullptr;
    b->ptried = false;
}

// the persistent kernel's context, when every instance qualifies (built from the instances' current
// argument blocks; rebuilt after any of them changed)
static void batch_persistent(ep_batch* b) {
    const int n = (int)b->h.size();
    std::vector<int> g(n);
    for (int i = 0; i < n; ++i) g[i] = b->h[i]->graph_gen;
    if (g != b->gens) {
        batch_drop(b);
        b->gens = g;
    }
    if (b->ptried) return;
    b->ptried = true;
    std::vector<const MixedCtx*> xs(n);
    for (int i = 0; i < n; ++i) {
        if (!b->h[i]->mixed) {
            b->pwhy = "FP64 instances run on the per-instance graphs";
            return;
        }
        xs[i] = &b->h[i]->mx;
    }
    b->pimpl = mixed_batch_create(xs.data(), n, &b->pwhy);
}

ep_status epgpu_batch_destroy(ep_batch* b) {
    if (!b) return EP_ERR_ARG;
    if (b->s) cudaStreamSynchronize(b->s);
    batch_drop(b);
    for (ep_handle* h : b->h) epgpu_destroy(h);
    if (b->dctl) cudaFree(b->dctl);
    if (b->dflags) cudaFree(b->dflags);
    if (b->hflags) cudaFreeHost(b->hflags);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->s) cudaStreamDestroy(b->s);
    delete b;
    return EP_OK;
}

ep_status epgpu_batch_create(int32_t n, const ep_cfg* cfg, const ep_cmpr* cmpr, const ep_mesh_view* mesh,
                             const int64_t* nmp, ep_batch** out) {
    g_create_error.clear();
    if (n <= 0 || !cfg || !cmpr || !mesh || !nmp || !out) return bfail(nullptr, EP_ERR_ARG, "null argument or n <= 0");
    *out = nullptr;
    ep_batch* b = new ep_batch();
    for (int i = 0; i < n; ++i) {
        ep_handle* h = nullptr;
        ep_status st = epgpu_create(&cfg[i], &cmpr[i], &mesh[i], nmp[i], &h);
        if (st != EP_OK) {
            std::string m = "instance " + std::to_string(i) + ": " + g_create_error;
            epgpu_batch_destroy(b);
            return bfail(nullptr, st, m);
        }
        b->h.push_back(h);
    }
    std::vector<Ctl*> c(n);
    for (int i = 0; i < n; ++i) c[i] = b->h[i]->ctl;
    cudaError_t e = cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->dctl, sizeof(Ctl*) * n);
    if (e == cudaSuccess) e = cudaMalloc(&b->dflags, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->hflags, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMemcpy(b->dctl, c.data(), sizeof(Ctl*) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e != cudaSuccess) {
        std::string m = std::string("batch create: ") + cudaGetErrorString(e);
        cudaGetLastError();
        epgpu_batch_destroy(b);
        return bfail(nullptr, EP_ERR_CUDA, m);
    }
    *out = b;
    return EP_OK;
}

const char* epgpu_batch_last_error(ep_batch* b) { return b ? b->err.c_str() : g_create_error.c_str(); }

ep_handle* epgpu_batch_instance(ep_batch* b, int32_t i) {
    if (!b || i < 0 || i >= (int)b->h.size()) return nullptr;
    return b->h[i];
}

ep_status epgpu_batch_upload(ep_batch* b, int32_t i, const ep_mpts_view* m) {
    if (!b || i < 0 || i >= (int)b->h.size()) return EP_ERR_ARG;
    ep_status st = epgpu_upload(b->h[i], m);
    if (st != EP_OK) return bfail(b, st, "instance " + std::to_string(i) + ": " + b->h[i]->err);
    return EP_OK;
}

ep_status epgpu_batch_download(ep_batch* b, int32_t i, ep_mpts_view* m) {
    if (!b || i < 0 || i >= (int)b->h.size()) return EP_ERR_ARG;
    cudaStreamSynchronize(b->s);
    ep_status st = epgpu_download(b->h[i], m);
    if (st != EP_OK) return bfail(b, st, "instance " + std::to_string(i) + ": " + b->h[i]->err);
    return EP_OK;
}

static ep_status batch_graph(ep_batch* b, int phase) {
    batch_persistent(b);
    if (b->exec[phase]) return EP_OK;
    const int n = (int)b->h.size();
    if (b->used_scheme() == 2) {
        cudaGraph_t g;
        BCK(b, cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal));
        mixed_batch_phase_steps(b->pimpl, phase == EP_PHASE_ELASTOPLASTIC, GRAPH_STEPS, b->tile, 0, b->s);
        mixed_batch_flags(b->pimpl, b->dflags, b->s);
        cudaError_t e = cudaStreamEndCapture(b->s, &g);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec[phase], g, 0);
        if (e == cudaSuccess) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return bfail(b, EP_ERR_CUDA, std::string("phase-kernel batch graph: ") + cudaGetErrorString(e));
        }
        return EP_OK;
    }
    if (b->used_scheme() == 1) {
        cudaGraph_t g;
        BCK(b, cudaGraphCreate(&g, 0));
        cudaError_t e = mixed_batch_graph(b->pimpl, phase == EP_PHASE_ELASTOPLASTIC, GRAPH_STEPS, b->tile, b->dflags, g);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec[phase], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return bfail(b, EP_ERR_CUDA, std::string("persistent batch graph: ") + cudaGetErrorString(e));
        }
        return EP_OK;
    }
    for (int i = 0; i < n; ++i) {
        ep_status st = build_graph(b->h[i], phase);
        if (st != EP_OK) return bfail(b, st, "instance " + std::to_string(i) + ": " + b->h[i]->err);
    }
    cudaGraph_t g;
    BCK(b, cudaGraphCreate(&g, 0));
    std::vector<cudaGraphNode_t> kids(n);
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < n && e == cudaSuccess; ++i)
        e = cudaGraphAddChildGraphNode(&kids[i], g, nullptr, 0, b->h[i]->graph_def[phase]);
    if (e == cudaSuccess) {
        cudaKernelNodeParams kp{};
        void* args[] = {(void*)&b->dctl, (void*)&n, (void*)&b->dflags};
        kp.func = (void*)k_batch_flags;
        kp.gridDim = dim3((n + 127) / 128);
        kp.blockDim = dim3(128);
        kp.sharedMemBytes = 0;
        kp.kernelParams = args;
        kp.extra = nullptr;
        cudaGraphNode_t fl;
        e = cudaGraphAddKernelNode(&fl, g, kids.data(), n, &kp);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec[phase], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bfail(b, EP_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
    }
    return EP_OK;
}

ep_status epgpu_batch_run(ep_batch* b, int32_t phase, double T, double tg, double* t_inout, int64_t* nsteps_out) {
    if (!b || !t_inout) return EP_ERR_ARG;
    if (phase != 0 && phase != 1) return bfail(b, EP_ERR_ARG, "phase must be 0 or 1");
    const int n = (int)b->h.size();
    ep_status st;
    for (int i = 0; i < n; ++i) {
        ep_handle* h = b->h[i];
        if (!h->uploaded) return bfail(b, EP_ERR_STATE, "instance " + std::to_string(i) + " not uploaded");
        if ((st = read_ctl(h)) != EP_OK) return bfail(b, st, h->err);
        if (h->hctl->err) {
            kernel_error(h);
            return bfail(b, (ep_status)h->hctl->err, "instance " + std::to_string(i) + ": " + h->err);
        }
        h->hctl->t = t_inout[i];
        h->hctl->T = T;
        h->hctl->tg = tg;
        h->hctl->phase = phase;
        h->hctl->active = 1;
        h->hctl->nsteps = 0;
        BCK(b, cudaMemcpyAsync(h->ctl, h->hctl, sizeof(Ctl), cudaMemcpyHostToDevice, h->s));
    }
    if ((st = batch_graph(b, phase)) != EP_OK) return st;
    for (ep_handle* h : b->h) BCK(b, cudaStreamSynchronize(h->s));
    BCK(b, cudaEventRecord(b->ev0, b->s));
    long long launched = 0;
    int failed = -1;
    while (true) {
        BCK(b, cudaGraphLaunch(b->exec[phase], b->s));
        ++launched;
        BCK(b, cudaMemcpyAsync(b->hflags, b->dflags, sizeof(int) * n, cudaMemcpyDeviceToHost, b->s));
        BCK(b, cudaStreamSynchronize(b->s));
        bool any = false;
        bool stuck = false;
        for (int i = 0; i < n; ++i) {
            if (b->hflags[i] & 2) failed = i;
            if (b->hflags[i] & 1) any = true;
            if (b->hflags[i] & 4) stuck = true;
        }
        if (stuck) return bfail(b, EP_ERR_TIMEOUT, "persistent batch kernel: a grid barrier wait gave up");
        if (failed >= 0 || !any) break;
        if (launched >= (1 << 24)) return bfail(b, EP_ERR_TIMEOUT, "batch time loop did not reach T");
    }
    BCK(b, cudaEventRecord(b->ev1, b->s));
    BCK(b, cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    b->last_ms = ms;
    for (int i = 0; i < n; ++i) {
        ep_handle* h = b->h[i];
        if ((st = read_ctl(h)) != EP_OK) return bfail(b, st, h->err);
        h->launches += launched * (b->used_scheme() != 0 ? 1 : h->graph_kernels[phase]);
        h->t = h->hctl->t;
        h->steps += h->hctl->nsteps;
        h->fresh = 0;
        t_inout[i] = h->hctl->t;
        if (nsteps_out) nsteps_out[i] = h->hctl->nsteps;
    }
    b->launches += launched;
    if (failed >= 0) {
        ep_handle* h = b->h[failed];
        st = kernel_error(h);
        return bfail(b, st == EP_OK ? EP_ERR_CUDA : st, "instance " + std::to_string(failed) + ": " + h->err);
    }
    return EP_OK;
}

// Tile-shape autotuner: time steps of dt = 0 (positions, velocities and stresses do not
// change; the lists are rebuilt with the same contents) of every instance with each P2G
// tile shape, keep the fastest for all instances.
ep_status epgpu_batch_autotune(ep_batch* b, int32_t phase, int32_t* tile_out, double* ms_out) {
    if (!b || (phase != 0 && phase != 1)) return EP_ERR_ARG;
    const int n = (int)b->h.size();
    const int tiles[3] = {16, 32, 64};
    double best = 1e300;
    int pick = 64;
    ep_status st;
    for (int i = 0; i < n; ++i) {
        ep_handle* h = b->h[i];
        if (!h->mixed) return bfail(b, EP_ERR_UNSUPPORTED, "the tile autotuner is for the mixed-precision step");
        if (h->rm_mode == EP_RMAP_LEARNED)
            return bfail(b, EP_ERR_STATE, "autotune with the exact return map (the network's outputs move states)");
        if ((st = read_ctl(h)) != EP_OK) return bfail(b, st, h->err);
        h->hctl->dt = 0.0;
        for (int k = 0; k < 3; ++k) h->hctl->g[k] = 0.0;
        h->hctl->phase = phase;
        h->hctl->active = 1;
        for (int k = 0; k < 3; ++k) h->hctl->vmax_bits[k] = 0ull;
        BCK(b, cudaMemcpyAsync(h->ctl, h->hctl, sizeof(Ctl), cudaMemcpyHostToDevice, h->s));
        BCK(b, cudaStreamSynchronize(h->s));
    }
    batch_persistent(b);
    int pick_scheme = 0;
    for (int k = 0; k < 9; ++k) b->tune_ms[k] = 0.0;
    // schemes timed: the instances' own step graphs (as child graphs of one batch graph) and, when
    // the batch qualifies for them, the persistent kernel and the phase kernels, each with the control
    // blocks as set above (the per-instance graphs can win: 2.10e9 against 1.87e9 particle-steps/s for
    // the phase kernels on a 48-instance draw of the ensemble)
    for (int sc = 0; sc < (b->pimpl ? 3 : 1); ++sc) {
        for (int c = 0; c < 3; ++c) {
            // scheme 0 as it runs: every instance's step (control kernel + mixed step with this tile)
            // captured as a child graph of one batch graph with no dependencies between them
            cudaGraphExec_t tg = nullptr;
            if (sc == 0) {
                cudaGraph_t g;
                BCK(b, cudaGraphCreate(&g, 0));
                cudaError_t e = cudaSuccess;
                for (size_t i = 0; i < b->h.size() && e == cudaSuccess; ++i) {
                    ep_handle* h = b->h[i];
                    MixedCtx mx = h->mx;
                    mx.p2g_tile = tiles[c];
                    mx.launches = nullptr;
                    mx.prof = nullptr;
                    cudaGraph_t hg;
                    e = cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal);
                    if (e == cudaSuccess) {
                        launch_ctl_begin_step(h->ctl, h->dim, b->s);
                        mixed_step(mx, phase, b->s);
                        e = cudaStreamEndCapture(b->s, &hg);
                    }
                    if (e == cudaSuccess) {
                        cudaGraphNode_t node;
                        e = cudaGraphAddChildGraphNode(&node, g, nullptr, 0, hg);
                        cudaGraphDestroy(hg);
                    }
                }
                if (e == cudaSuccess) e = cudaGraphInstantiate(&tg, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    cudaGetLastError();
                    return bfail(b, EP_ERR_CUDA, std::string("autotune graph: ") + cudaGetErrorString(e));
                }
            }
            for (int rep = 0; rep < 4; ++rep) {
                if (rep == 1) BCK(b, cudaEventRecord(b->ev0, b->s));
                if (sc == 1) BCK(b, mixed_batch_launch(b->pimpl, phase == EP_PHASE_ELASTOPLASTIC, 1, tiles[c], 1, b->s));
                else if (sc == 2) mixed_batch_phase_steps(b->pimpl, phase == EP_PHASE_ELASTOPLASTIC, 1, tiles[c], 1, b->s);
                else BCK(b, cudaGraphLaunch(tg, b->s));
            }
            BCK(b, cudaGetLastError());
            if (tg) {
                BCK(b, cudaStreamSynchronize(b->s));
                cudaGraphExecDestroy(tg);
            }
            BCK(b, cudaEventRecord(b->ev1, b->s));
            BCK(b, cudaEventSynchronize(b->ev1));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, b->ev0, b->ev1);
            b->tune_ms[3 * sc + c] = ms / 3.0;
            if (ms < best) {
                best = ms;
                pick = tiles[c];
                pick_scheme = sc;
            }
        }
    }
    if (ms_out)
        for (int c = 0; c < 3; ++c) ms_out[c] = b->tune_ms[3 * pick_scheme + c];
    for (ep_handle* h : b->h) {
        if ((st = read_ctl(h)) != EP_OK) return bfail(b, st, h->err);
        if (h->hctl->err) {
            kernel_error(h);
            return bfail(b, (ep_status)h->hctl->err, h->err);
        }
        h->mx.p2g_tile = pick;
        drop_graphs(h);
    }
    if (b->pimpl && mixed_batch_error(b->pimpl)) return bfail(b, EP_ERR_TIMEOUT, "persistent batch kernel: a grid barrier wait gave up");
    batch_drop(b);
    b->tile = pick;
    b->scheme = pick_scheme;
    if (tile_out) *tile_out = pick;
    return EP_OK;
}

int32_t epgpu_batch_scheme(ep_batch* b) {
    if (!b) return -1;
    batch_persistent(b);
    return b->used_scheme();
}

ep_status epgpu_batch_set_scheme(ep_batch* b, int32_t scheme) {
    if (!b || scheme < -1 || scheme > 2) return EP_ERR_ARG;
    batch_persistent(b);
    if (scheme >= 1 && !b->pimpl) return bfail(b, EP_ERR_UNSUPPORTED, "batch kernels over all instances: " + b->pwhy);
    for (int k = 0; k < 2; ++k)
        if (b->exec[k]) {
            cudaGraphExecDestroy(b->exec[k]);
            b->exec[k] = nullptr;
        }
    b->scheme = scheme;
    return EP_OK;
}

ep_status epgpu_batch_tuning(ep_batch* b, double* ms9, int32_t* persistent_available) {
    if (!b || !ms9) return EP_ERR_ARG;
    batch_persistent(b);
    for (int k = 0; k < 9; ++k) ms9[k] = b->tune_ms[k];
    if (persistent_available) *persistent_available = b->pimpl ? 1 : 0;
    return EP_OK;
}

ep_status epgpu_batch_stats(ep_batch* b, double* device_ms, int64_t* graph_launches) {
    if (!b) return EP_ERR_ARG;
    if (device_ms) *device_ms = b->last_ms;
    if (graph_launches) *graph_launches = b->launches;
    return EP_OK;
}

}  // extern "C"
