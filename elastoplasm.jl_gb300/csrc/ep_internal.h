// ep_internal.h -- host-side launchers shared between the translation units.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "ep_dev.cuh"
#include "ep_mixed.cuh"

struct ep_mlp;   // learned return map object (include/epgpu.h)

namespace ep {

// CUDA-event timers between consecutive kernels of a step (profiling mode).
struct Prof {
    bool on = false;
    int n = 0;
    std::vector<cudaEvent_t> ev;
    std::vector<const char*> name;
    std::map<std::string, std::pair<long long, double>> acc;
    void begin(cudaStream_t s) {
        n = 0;
        mark("begin", s);
    }
    // the events made ahead (a capture records into them without creating any)
    void reserve(int k) {
        while ((int)ev.size() < k) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return;
            ev.push_back(e);
            name.push_back(nullptr);
        }
    }
    void mark(const char* nm, cudaStream_t s) {
        if (!on) return;
        if (n >= (int)ev.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ev.push_back(e);
            name.push_back(nullptr);
        }
        // inside a stream capture (the profiled step graph) the record must be a node of the graph
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(s, &cs);
        if (cs == cudaStreamCaptureStatusActive) cudaEventRecordWithFlags(ev[n], s, cudaEventRecordExternal);
        else cudaEventRecord(ev[n], s);
        name[n] = nm;
        ++n;
    }
    // after the stream was synchronised
    void collect() {
        if (!on) return;
        for (int i = 1; i < n; ++i) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[i - 1], ev[i]);
            auto& a = acc[name[i]];
            a.first += 1;
            a.second += ms;
        }
        n = 0;
    }
    ~Prof() {
        for (auto e : ev) cudaEventDestroy(e);
    }
};

// Exclusive prefix sum of in[0..n) into out[0..n]; out[n] = total.  `tmp`
// must hold scan_tmp_ints(n) ints.  Works in place (in == out) too.
int scan_tmp_ints(int n);
void launch_exclusive_scan(const int* in, int* out, int n, int* tmp, cudaStream_t s);

// Sort every segment data[start[i]..start[i+1]) ascending (warp per segment).
void launch_segsort(const int* start, int nseg, int* data, cudaStream_t s);

// Counting-sort placement of points into cells: cell_list[cell_start[c] + k]
// for the k-th point of cell c seen by the atomic cursor (order fixed by the
// following launch_segsort).
void launch_place_cells(const int* p2e, int np, const int* cell_start, int* cursor, int* cell_list,
                        const Ctl* ctl, cudaStream_t s);

// Point -> cell (the reference's clamp(fld(x - x0, h), 0, nel-1), tplgy.jl:43-96)
// with a per-cell count; x is dim arrays of np doubles.
void launch_bin_points(const Geo& g, const double* const* x, int np, int* p2e, int* cell_count,
                       Ctl* ctl, cudaStream_t s);

// Message returned by epgpu_last_error(NULL) for calls without a handle (ep_api.cu).
void set_global_error(const char* msg);

// FP64 step launchers (ep_fp64.cu)
struct Fp64Ctx {
    Cfg cf;
    Geo g;
    Mat mt;
    Ctl* ctl;
    P64 P;
    N64 N;
    Sort S;
    int np;
    long long* launches;
    Prof* prof;
};
void fp64_step(const Fp64Ctx& c, int phase, cudaStream_t s);
void fp64_check_finite(const Fp64Ctx& c, cudaStream_t s);

// mixed-precision step (ep_mixed.cu)
struct MixedCtx {
    void* impl;               // host image of the kernels' argument block (MCtx)
    ep_mlp* net;              // learned return map (EP_RMAP_LEARNED) or nullptr
    void* grid_zero;          // node accumulators zeroed at each step start
    size_t grid_zero_bytes;
    void* sort_zero;          // both parities' cell counts and the cursor
    size_t sort_zero_bytes;
    int* scan_in;
    int* scan_out;
    Prof* prof;
    long long* launches;
    int p2g_tile;             // cells per CTA of the P2G kernel: 16, 32 or 64 (autotuned)
    int begin_step = 0;       // 1: the step's first kernel also starts the step (k_ctl_begin_step's work)
    // host-loop overlap (epgpu_step_fields): recorded once the G2P has written the step's positions and
    // velocities, and waited for before the constitutive pass (whose other inputs arrive meanwhile)
    cudaEvent_t ev_moved = nullptr;
    cudaEvent_t ev_need = nullptr;
    bool hooks_internal = false;      // in a capture: fork / join events of that capture, not external nodes
};
// Host point arrays, page-locked and mapped (their device-accessible addresses), in the reference's
// column-major layout (k components per point): the direct transfers of the mixed precisions, which
// convert between these and the step's own layout in one pass, without the FP64 staging layout.
struct HostAoS {
    double *x, *v, *l, *F, *b, *tau, *sig, *ep, *dlam, *dv;
};
// the arrays a direct transfer can move (EP_MPTS_* bits; an upload must include the positions)
constexpr uint64_t MIXED_DIRECT_FIELDS = EP_MPTS_X | EP_MPTS_V | EP_MPTS_L | EP_MPTS_FIJ | EP_MPTS_BIJ | EP_MPTS_TAU |
                                         EP_MPTS_SIG | EP_MPTS_EPII | EP_MPTS_DLAM | EP_MPTS_DVIJ;
// host arrays in `mask` -> the mixed layout, and the cell lists rebuilt from the host positions
// (bin = false: the arrays of the mask only, positions and cell lists untouched)
void mixed_import_host(const MixedCtx& X, const HostAoS& H, uint64_t mask, cudaStream_t s, bool bin = true);
// the mixed layout -> the host arrays in `mask`
// (par >= 0: the offsets of that parity, for x and v right after the G2P of a running step)
void mixed_export_host(const MixedCtx& X, const HostAoS& H, uint64_t mask, cudaStream_t s, int par = -1);
size_t mixed_ctx_size();
// persistent batch kernel over n 2d mixed instances (nullptr + reason when the batch is not eligible)
void* mixed_batch_create(const MixedCtx* const* xs, int n, std::string* why);
void mixed_batch_destroy(void* b);
cudaError_t mixed_batch_graph(void* b, int plastic, int steps, int tile, int* dflags, cudaGraph_t g);
cudaError_t mixed_batch_launch(void* b, int plastic, int steps, int tile, int keep_ctl, cudaStream_t s);
int mixed_batch_error(void* b);
void mixed_batch_phase_steps(void* b, int plastic, int steps, int tile, int keep_ctl, cudaStream_t s);
void mixed_batch_flags(void* b, int* dflags, cudaStream_t s);
void mixed_ctx_init(void* mem, const Cfg& cf, const Geo& g, Ctl* ctl, const PM& P, const NM& N, const SM& S,
                    const double* Del, const double* Cmp, double Kc, double Gc, double Hp, double c, int acc);
void mixed_step(const MixedCtx& X, int phase, cudaStream_t s);
// return map of the mixed step: mode EP_RMAP_*, slot buffers of the learned mode
// (features, outputs, aux, point ids, slot count) or the record buffer of the network
struct RmapBufs {
    int mode;
    float *rx, *ry, *raux;
    int* rpt;
    int* rcount;
    int* fbcount;
    int* fblist;
    long long* rec_count;
    long long rec_cap;
};
void mixed_set_rmap(void* impl, const RmapBufs& b);
// deterministic mode buffers: per-cell node partials (ncell x 16 x 5) and one float per point
void mixed_set_det(void* impl, float* part, float* ptmp);
// network kernels used by the step (ep_mlp.cu)
void mlp_infer(ep_mlp* m, const float* X, const int* ndev, int cap, float* Y, cudaStream_t s);
float* mlp_record_x(ep_mlp* m);
float* mlp_record_t(ep_mlp* m);
long long* mlp_record_count(ep_mlp* m);
long long mlp_record_cap(ep_mlp* m);
void launch_mixed_scan(const MixedCtx& X, cudaStream_t s);
void mixed_initial_scan(const MixedCtx& X, cudaStream_t s);
// the staging fields in `mask` (EP_MPTS_* bits) into the mixed layout, then the cell lists rebuilt from
// the staging positions (which must be current)
void mixed_import(const MixedCtx& X, const P64& Q, cudaStream_t s, uint64_t mask = EP_MPTS_ALL);
// the FP64 staging state from the mixed state: the point arrays in `mask` (need_eps = false skips the
// log strain ϵ = ½ log b) and, with `nodes`, the nodal fields of the last step
void mixed_export(const MixedCtx& X, const P64& Q, const N64& QN, cudaStream_t s, bool need_eps = true,
                  uint64_t mask = EP_MPTS_ALL, bool nodes = true);

// control-block kernels (ep_fp64.cu)
void launch_ctl_begin_run(Ctl* ctl, const Geo& g, double c, cudaStream_t s);
void launch_ctl_begin_step(Ctl* ctl, int dim, cudaStream_t s);
void launch_ctl_set_step(Ctl* ctl, double dt, const double* g, int phase, cudaStream_t s);
void launch_ctl_end(Ctl* ctl, cudaStream_t s);

}  // namespace ep
