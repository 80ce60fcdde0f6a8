// ep_sort.cu -- particle binning as a stable, bit-exact counting sort.
//
// The reference assigns each point to a cell (p2e2n_{2,3}d, tplgy.jl:43-96)
// and later walks cells' point lists in ascending point order (the sparse
// e2p/p2p bookkeeping of nonlocal.jl:18-47).  Here: count points per cell
// with atomics, exclusive-scan the counts, place each point with an atomic
// cursor, then sort every cell's segment by point id (warp bitonic sort), so
// the result is independent of atomic arrival order: a stable counting sort.
#include <atomic>
#include <climits>
#include <cstdio>

#include "../../include/epgpu.h"
#include "ep_internal.h"

namespace ep {

constexpr int SCAN_BS = 1024;
constexpr int SCAN_IPT = 4;
constexpr int SCAN_CHUNK = SCAN_BS * SCAN_IPT;

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total in *tot.
// ws[0..31] hold the per-warp exclusive offsets, ws[32] the block total.
__device__ __forceinline__ int block_excl_scan(int v, int* tot) {
    __shared__ int ws[33];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int inc = warp_incl_scan(v);
    if (lane == 31) ws[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int s = lane < nw ? ws[lane] : 0;
        int si = warp_incl_scan(s);
        if (lane < nw) ws[lane] = si - s;
        if (lane == 31) ws[32] = si;   // lanes >= nw add 0, so lane 31 holds the total
    }
    __syncthreads();
    int r = ws[wid] + inc - v;
    *tot = ws[32];
    __syncthreads();
    return r;
}

__global__ void k_scan_local(const int* __restrict__ in, int* out, int* bsum, int n) {
    const int base = blockIdx.x * SCAN_CHUNK + threadIdx.x * SCAN_IPT;
    int v[SCAN_IPT];
    int s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; ++i) {
        v[i] = (base + i < n) ? in[base + i] : 0;
        s += v[i];
    }
    int tot;
    int ex = block_excl_scan(s, &tot);
#pragma unroll
    for (int i = 0; i < SCAN_IPT; ++i) {
        if (base + i < n) out[base + i] = ex;
        ex += v[i];
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void k_scan_sums(int* bsum, int nb, int* out, int n) {
    // one block: exclusive scan of nb <= SCAN_CHUNK block totals
    const int base = threadIdx.x * SCAN_IPT;
    int v[SCAN_IPT];
    int s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; ++i) {
        v[i] = (base + i < nb) ? bsum[base + i] : 0;
        s += v[i];
    }
    int tot;
    int ex = block_excl_scan(s, &tot);
#pragma unroll
    for (int i = 0; i < SCAN_IPT; ++i) {
        if (base + i < nb) bsum[base + i] = ex;
        ex += v[i];
    }
    if (threadIdx.x == 0) out[n] = tot;
}

__global__ void k_scan_add(int* out, const int* bsum, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += bsum[i / SCAN_CHUNK];
}

int scan_tmp_ints(int n) { return (n + SCAN_CHUNK - 1) / SCAN_CHUNK + 1; }

void launch_exclusive_scan(const int* in, int* out, int n, int* tmp, cudaStream_t s) {
    int nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    if (nb == 0) {
        cudaMemsetAsync(out, 0, sizeof(int), s);
        return;
    }
    // n up to SCAN_CHUNK^2 (16.7 M) elements; the callers check the bound
    k_scan_local<<<nb, SCAN_BS, 0, s>>>(in, out, tmp, n);
    k_scan_sums<<<1, SCAN_BS, 0, s>>>(tmp, nb, out, n);
    if (nb > 1) k_scan_add<<<(n + 255) / 256, 256, 0, s>>>(out, tmp, n);
}

// ---------------------------------------------------------------------------
// Segmented sort: one warp per segment.  <= 32 elements: bitonic network in
// registers; <= 1024: bitonic network in shared memory; longer: serial
// insertion sort by one lane (only for pathological pile-ups).
// ---------------------------------------------------------------------------
constexpr int SEG_WARPS = 8;
constexpr int SEG_SMEM = 1024;

__global__ void __launch_bounds__(SEG_WARPS * 32) k_segsort(const int* __restrict__ start, int nseg, int* data) {
    __shared__ int buf[SEG_WARPS][SEG_SMEM];
    const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
    const int seg = blockIdx.x * SEG_WARPS + wb;
    if (seg >= nseg) return;
    const int b = start[seg], L = start[seg + 1] - b;
    if (L <= 1) return;
    if (L <= 32) {
        int v = lane < L ? data[b + lane] : INT_MAX;
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                int o = __shfl_xor_sync(0xffffffffu, v, j);
                bool asc = (lane & k) == 0;
                bool low = (lane & j) == 0;
                v = (low == asc) ? min(v, o) : max(v, o);
            }
        if (lane < L) data[b + lane] = v;
        return;
    }
    if (L <= SEG_SMEM) {
        int P = 64;
        while (P < L) P <<= 1;
        int* s = buf[wb];
        for (int i = lane; i < P; i += 32) s[i] = i < L ? data[b + i] : INT_MAX;
        __syncwarp();
        for (int k = 2; k <= P; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = lane; i < P; i += 32) {
                    int q = i ^ j;
                    if (q > i) {
                        int a = s[i], c = s[q];
                        bool asc = (i & k) == 0;
                        if ((a > c) == asc) { s[i] = c; s[q] = a; }
                    }
                }
                __syncwarp();
            }
        for (int i = lane; i < L; i += 32) data[b + i] = s[i];
        return;
    }
    if (lane == 0) {
        for (int i = 1; i < L; ++i) {
            int v = data[b + i];
            int j = i - 1;
            while (j >= 0 && data[b + j] > v) {
                data[b + j + 1] = data[b + j];
                --j;
            }
            data[b + j + 1] = v;
        }
    }
}

void launch_segsort(const int* start, int nseg, int* data, cudaStream_t s) {
    if (nseg <= 0) return;
    k_segsort<<<(nseg + SEG_WARPS - 1) / SEG_WARPS, SEG_WARPS * 32, 0, s>>>(start, nseg, data);
}

__global__ void k_place_cells(const int* __restrict__ p2e, int np, const int* __restrict__ cell_start, int* cursor,
                              int* cell_list, const Ctl* ctl) {
    if (ctl && !ctl->active) return;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    int c = p2e[p];
    if (c < 0) return;
    int k = atomicAdd(&cursor[c], 1);
    int pos = cell_start[c] + k;
    if (pos < cell_start[c + 1]) cell_list[pos] = p;      // counts and placements always agree;
    else if (ctl) set_err(const_cast<Ctl*>(ctl), EP_ERR_CUDA, p);   // guard against a corrupt scan
}

void launch_place_cells(const int* p2e, int np, const int* cell_start, int* cursor, int* cell_list, const Ctl* ctl,
                        cudaStream_t s) {
    if (np <= 0) return;
    k_place_cells<<<(np + 255) / 256, 256, 0, s>>>(p2e, np, cell_start, cursor, cell_list, ctl);
}

template <int D>
__global__ void k_bin_points(Geo g, const double* __restrict__ x0, const double* __restrict__ x1,
                             const double* __restrict__ x2, int np, int* p2e, int* cell_count, Ctl* ctl) {
    if (ctl && !ctl->active) return;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    double xp[3] = {x0[p], x1[p], D == 3 ? x2[p] : 0.0};
    int e[3];
    int c = cell_index<D>(xp, g, e);
    p2e[p] = c;
    if (c >= 0) atomicAdd(&cell_count[c], 1);
    else if (ctl) set_err(ctl, EP_ERR_NONFINITE, p);
}

void launch_bin_points(const Geo& g, const double* const* x, int np, int* p2e, int* cell_count, Ctl* ctl,
                       cudaStream_t s) {
    if (np <= 0) return;
    int nb = (np + 255) / 256;
    if (g.dim == 2) k_bin_points<2><<<nb, 256, 0, s>>>(g, x[0], x[1], nullptr, np, p2e, cell_count, ctl);
    else k_bin_points<3><<<nb, 256, 0, s>>>(g, x[0], x[1], x[2], np, p2e, cell_count, ctl);
}

}  // namespace ep

// ---------------------------------------------------------------------------
// Stand-alone C-ABI binning (include/epgpu.h).
// ---------------------------------------------------------------------------
extern "C" ep_status epgpu_bin_cells(int32_t dim, const int64_t* nel, const double* h, const double* x0,
                                     const double* x_dev, int64_t nmp, int32_t* p2e_dev, int32_t* cell_start_dev,
                                     int32_t* cell_list_dev, void* stream) {
    using namespace ep;
    if ((dim != 2 && dim != 3) || !nel || !h || !x0 || nmp < 0) return EP_ERR_ARG;
    if (nmp > 0 && (!x_dev || !p2e_dev || !cell_list_dev)) return EP_ERR_ARG;
    if (!cell_start_dev) return EP_ERR_ARG;
    long long ncell = 1;
    for (int d = 0; d < dim; ++d) {
        if (nel[d] <= 0 || !(h[d] > 0.0)) return EP_ERR_ARG;
        ncell *= nel[d];
    }
    if (ncell > (long long)SCAN_CHUNK * SCAN_CHUNK || nmp > INT_MAX) return EP_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    Geo g{};
    g.dim = dim;
    for (int d = 0; d < dim; ++d) {
        g.nel[d] = (int)nel[d];
        g.h[d] = h[d];
        g.x0[d] = x0[d];
    }
    g.ncell = (int)ncell;
    const int np = (int)nmp;
    const int nc = (int)ncell;
    // scratch: per-cell counters/cursors and the scan's block totals
    size_t n_tmp = (size_t)scan_tmp_ints(nc);
    int* scratch = nullptr;
    if (cudaMallocAsync((void**)&scratch, sizeof(int) * (2 * (size_t)nc + n_tmp), s) != cudaSuccess) {
        cudaGetLastError();
        return EP_ERR_NOMEM;
    }
    int* count = scratch;
    int* cursor = scratch + nc;
    int* tmp = scratch + 2 * (size_t)nc;
    cudaMemsetAsync(scratch, 0, sizeof(int) * 2 * (size_t)nc, s);
    const double* xs[3] = {x_dev, x_dev + nmp, dim == 3 ? x_dev + 2 * nmp : nullptr};
    launch_bin_points(g, xs, np, p2e_dev, count, nullptr, s);
    launch_exclusive_scan(count, cell_start_dev, nc, tmp, s);
    launch_place_cells(p2e_dev, np, cell_start_dev, cursor, cell_list_dev, nullptr, s);
    launch_segsort(cell_start_dev, nc, cell_list_dev, s);
    cudaFreeAsync(scratch, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return EP_ERR_CUDA;
    e = cudaGetLastError();
    return e == cudaSuccess ? EP_OK : EP_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the stand-alone binning (include/epgpu.h).
// Its scratch -- per-cell counters, per-cell cursors and the scan's block
// totals -- is this file-scope device array, sized for EPGPU_NOALLOC_MAX_CELLS
// cells.  Host code must not pass `g_bin_scratch` itself to a kernel (on the
// host the name is only a stand-in, not a device address): the device address
// is looked up with cudaGetSymbolAddress on every call, with the caller's
// device current.  The lookup is a host-side table read once the module is
// loaded, and a per-call lookup stays valid across a cudaDeviceReset or a
// primary context that was released and created again (a cached address
// would then point into the freed module).
// ---------------------------------------------------------------------------
namespace {

constexpr int NOALLOC_TMP_INTS = (EPGPU_NOALLOC_MAX_CELLS + ep::SCAN_CHUNK - 1) / ep::SCAN_CHUNK + 1;
constexpr int NOALLOC_SCRATCH_INTS = 2 * EPGPU_NOALLOC_MAX_CELLS + NOALLOC_TMP_INTS;

static __device__ __align__(256) int g_bin_scratch[NOALLOC_SCRATCH_INTS];

// Device address of g_bin_scratch in the current context.
cudaError_t noalloc_scratch(int** out) {
    void* q = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&q, g_bin_scratch);
    if (e != cudaSuccess) return e;
    *out = (int*)q;
    return cudaSuccess;
}

}  // namespace

extern "C" ep_status epgpu_bin_cells_noalloc(int32_t dim, const int64_t* nel, const double* h, const double* x0,
                                             const double* x_dev, int64_t nmp, int32_t* p2e_dev,
                                             int32_t* cell_start_dev, int32_t* cell_list_dev, void* stream) {
    using namespace ep;
    if ((dim != 2 && dim != 3) || !nel || !h || !x0 || nmp < 0) return EP_ERR_ARG;
    if (nmp > 0 && (!x_dev || !p2e_dev || !cell_list_dev)) return EP_ERR_ARG;
    if (!cell_start_dev) return EP_ERR_ARG;
    long long ncell = 1;
    for (int d = 0; d < dim; ++d) {
        if (nel[d] <= 0 || !(h[d] > 0.0)) return EP_ERR_ARG;
        ncell *= nel[d];
        if (ncell > EPGPU_NOALLOC_MAX_CELLS) break;
    }
    if (ncell > EPGPU_NOALLOC_MAX_CELLS) {
        char msg[160];
        snprintf(msg, sizeof msg,
                 "epgpu_bin_cells_noalloc: the mesh has more than the %d cells its static scratch holds; "
                 "use epgpu_bin_cells", EPGPU_NOALLOC_MAX_CELLS);
        set_global_error(msg);
        return EP_ERR_ARG;
    }
    if (nmp > INT_MAX) return EP_ERR_ARG;
    int* scratch = nullptr;
    cudaError_t e = noalloc_scratch(&scratch);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_global_error("epgpu_bin_cells_noalloc: cudaGetSymbolAddress of the static scratch failed");
        return EP_ERR_CUDA;
    }
    cudaStream_t s = (cudaStream_t)stream;
    Geo g{};
    g.dim = dim;
    for (int d = 0; d < dim; ++d) {
        g.nel[d] = (int)nel[d];
        g.h[d] = h[d];
        g.x0[d] = x0[d];
    }
    g.ncell = (int)ncell;
    const int np = (int)nmp;
    const int nc = (int)ncell;
    int* count = scratch;
    int* cursor = scratch + nc;
    int* tmp = scratch + 2 * (size_t)nc;
    // the array keeps the previous call's contents: clear the counters and cursors
    cudaMemsetAsync(scratch, 0, sizeof(int) * 2 * (size_t)nc, s);
    const double* xs[3] = {x_dev, x_dev + nmp, dim == 3 ? x_dev + 2 * nmp : nullptr};
    launch_bin_points(g, xs, np, p2e_dev, count, nullptr, s);
    launch_exclusive_scan(count, cell_start_dev, nc, tmp, s);
    launch_place_cells(p2e_dev, np, cell_start_dev, cursor, cell_list_dev, nullptr, s);
    launch_segsort(cell_start_dev, nc, cell_list_dev, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return EP_ERR_CUDA;
    e = cudaGetLastError();
    return e == cudaSuccess ? EP_OK : EP_ERR_CUDA;
}
