// ep_mlp.cu -- the learned return map: a 6 -> 128 x 4 (SiLU) -> 3 MLP on the
// tensor cores (tcgen05, BF16 operands, FP32 accumulation in tensor memory),
// its training kernels (backward GEMMs, MSE loss, Adam) and the C ABI of the
// network object.
//
// There is no counterpart in the reference: the network is a surrogate of the
// finite-strain Drucker-Prager return (elast.jl:51-54, DP.jl:33-66) in the
// principal-space form of ep_rmap.h, trained on pairs the exact map emits.
//
// Layer l computes Z_l = H_{l-1} W_l^T + b_l (W_l stored out x in, row-major),
// H_l = SiLU(Z_l) for l = 1..4, Y = H_4 W_5^T + b_5.  Operands are BF16; Z, the
// outputs and every gradient accumulate in FP32.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/epgpu.h"
#include "ep_internal.h"
#include "ep_rmap.h"
#include "ep_tc.cuh"

namespace ep {
namespace mlp {

constexpr int W = 128;        // hidden width
constexpr int KIN = 16;       // input features padded to one K step
constexpr int NO = 16;        // outputs padded to the smallest N of an M = 128 MMA
constexpr int NIN = 6, NOUT = 3;
constexpr int MT = 128;       // rows per tile
// FP32 master parameters, W row-major (out x in)
constexpr int OW1 = 0, OB1 = OW1 + W * NIN;
constexpr int OW2 = OB1 + W, OB2 = OW2 + W * W;
constexpr int OW3 = OB2 + W, OB3 = OW3 + W * W;
constexpr int OW4 = OB3 + W, OB4 = OW4 + W * W;
constexpr int OW5 = OB4 + W, OB5 = OW5 + NOUT * W;
constexpr int NPARAM = OB5 + NOUT;
static_assert(NPARAM == EP_MLP_NPARAM, "parameter count");
// packed BF16 image of the forward kernel (K-major canonical operands) + FP32 biases
constexpr int IW1 = 0, IW2 = IW1 + W * KIN * 2, IW3 = IW2 + W * W * 2, IW4 = IW3 + W * W * 2;
constexpr int IW5 = IW4 + W * W * 2, IBIAS = IW5 + NO * W * 2;
constexpr int IMG_BYTES = IBIAS + (4 * W + NO) * 4;
static_assert(IMG_BYTES % 16 == 0, "bulk copy size");

__host__ __device__ constexpr int w_off(int l) { return l == 1 ? OW1 : l == 2 ? OW2 : l == 3 ? OW3 : l == 4 ? OW4 : OW5; }
__host__ __device__ constexpr int b_off(int l) { return l == 1 ? OB1 : l == 2 ? OB2 : l == 3 ? OB3 : l == 4 ? OB4 : OB5; }
__host__ __device__ constexpr int n_in(int l) { return l == 1 ? NIN : W; }
__host__ __device__ constexpr int n_out(int l) { return l == 5 ? NOUT : W; }

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}
// SiLU through the hardware tanh: silu(z) = z sigmoid(z), sigmoid(z) = (1 + tanh(z / 2)) / 2.
// tanh.approx has a relative error near 2^-11, below the BF16 rounding of the activations.
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float silu(float z) {
    const float hz = 0.5f * z;
    return fmaf(hz, tanh_approx(hz), hz);
}
__device__ __forceinline__ float dsilu(float z) {
    const float s = fmaf(0.5f, tanh_approx(0.5f * z), 0.5f);
    return s * (1.f + z * (1.f - s));
}

// named barriers of one NT-thread group (ids 1 .. ; 0 is __syncthreads)
template <int NT>
__device__ __forceinline__ void grp_sync(int id) { asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(NT) : "memory"); }
template <int NT>
__device__ __forceinline__ bool grp_sync_and(int id, bool v) {
    int r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.s32 p, %1, 0;\n\tbar.red.and.pred q, %2, %3, p;\n\tselp.s32 %0, 1, 0, q;\n\t}"
                 : "=r"(r)
                 : "r"((int)v), "r"(id), "n"(NT)
                 : "memory");
    return r != 0;
}

// ---------------------------------------------------------------------------
// forward, fused over the five layers; one CTA (32 warps) per SM, FWD_GROUPS = 2 groups of
// FWD_GW = 16 warps each walking its own tiles of 128 rows, so that the groups' epilogues overlap
// each other's MMAs.  Warp w of a group reads TMEM lanes 32 (w % 4) .. + 31 (its rows) and the
// column quarter (w % 16) / 4 of every accumulator of its group (32 columns: two 16-column loads
// per layer and thread).  The step's launches hold a tile or two per CTA, so the epilogue of one
// tile is the critical path: 16 warps per tile halve it against 8.
struct FwdArgs {
    const float* X;       // rows of RM_NX floats (the first 6 are the inputs)
    int n;                // rows, or (ndev != nullptr) the capacity
    const int* ndev;      // device row count (in-step use)
    float* Y;             // rows of RM_NY floats (3 outputs, slot 3 = 0)
    const uint8_t* img;   // packed weights (IMG_BYTES, 16-byte aligned)
    __nv_bfloat16* Hst;   // training: H0 (n x 16), H1..H4 (n x 128), BF16
    float* Zst;           // training: Z1..Z4 (n x 128)
    int* err;             // set to 1 when a wait times out
};

// FWD_GROUPS 128-row tiles in flight per CTA: group g (warps FWD_GW g .. FWD_GW (g + 1) - 1) owns
// activation buffer FWD_SH + g and input buffer FWD_SX + g, the hidden-layer accumulator in TMEM
// columns 128 g .. 128 g + 127, the output accumulator in columns 384 + 32 g .. + 15, and mbarrier
// 1 + g; the weights are shared
constexpr int FWD_GROUPS = 2;
constexpr int FWD_GW = 16;                     // warps per group (a multiple of 4: the TMEM lane quarters)
constexpr int FWD_GT = 32 * FWD_GW;            // threads per group
constexpr int FWD_COLS = W / (FWD_GW / 4);     // accumulator columns of one warp
constexpr int FWD_SH = 0, FWD_SX = FWD_SH + FWD_GROUPS * MT * W * 2, FWD_SW = FWD_SX + FWD_GROUPS * MT * KIN * 2;
constexpr int FWD_BAR = FWD_SW + IMG_BYTES, FWD_SMEM = FWD_BAR + 48;
static_assert(FWD_SW % 128 == 0 && FWD_BAR % 8 == 0, "shared layout alignment");
static_assert(FWD_SMEM <= 232448, "shared memory of one CTA");
static_assert(128 * FWD_GROUPS <= 384 && 384 + 32 * FWD_GROUPS <= 512, "TMEM columns of the groups");

constexpr int FWD_THREADS = FWD_GT * FWD_GROUPS;
static_assert(FWD_THREADS <= 1024 && FWD_COLS % 16 == 0 && FWD_GT >= MT, "group shape");

__global__ void __launch_bounds__(FWD_THREADS, 1) km_mlp_fwd(FwdArgs a) {
    extern __shared__ __align__(128) uint8_t sm[];
    uint8_t* sW = sm + FWD_SW;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + FWD_BAR);       // [0] weights, [1 + g] group g's MMAs
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + FWD_BAR + 8 * (1 + FWD_GROUPS));
    const int n = a.ndev ? min(*a.ndev, a.n) : a.n;
    const int ntiles = (n + MT - 1) / MT;
    if (FWD_GROUPS * (int)blockIdx.x >= ntiles) return;     // the whole CTA, before any shared state
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int i = 0; i <= FWD_GROUPS; ++i) tc::mbar_init(&bar[i], 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tslot, 512);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tall = *tslot;
    if (tid == 0) {
        tc::mbar_arrive_expect_tx(&bar[0], IMG_BYTES);
        for (int o = 0; o < IMG_BYTES; o += 32768) {
            const int b = min(32768, IMG_BYTES - o);
            tc::bulk_g2s(sW + o, a.img + o, (uint32_t)b, &bar[0]);
        }
    }
    bool ok = tc::mbar_wait(&bar[0], 0);
    ok = __syncthreads_and(ok);
    // group g: its own tiles, buffers, accumulator columns and barrier; the two groups' MMAs
    // queue on the tensor core while the other group runs its epilogue
    const int g = warp / FWD_GW, gt = tid % FWD_GT, gw = warp % FWD_GW;
    uint8_t* sH = sm + FWD_SH + g * (MT * W * 2);
    uint8_t* sX = sm + FWD_SX + g * (MT * KIN * 2);
    uint64_t* gbar = &bar[1 + g];
    const uint32_t tbase = tall + (uint32_t)(128 * g);             // hidden layers
    const uint32_t tout = tall + (uint32_t)(384 + 32 * g);         // output layer
    const float* bias = reinterpret_cast<const float*>(sW + IBIAS);
    const uint32_t aX = tc::smem_u32(sX), aH = tc::smem_u32(sH), aW = tc::smem_u32(sW);
    const uint32_t id128 = tc::idesc_bf16(MT, W), id16 = tc::idesc_bf16(MT, NO);
    const int q = gw & 3, ch = gw >> 2;            // lane quarter, column block (FWD_COLS columns)
    const int row = 32 * q + lane;
    const uint32_t trow = tbase + ((uint32_t)(32 * q) << 16);
    uint32_t ph = 0;
    for (int tile = FWD_GROUPS * blockIdx.x + g; ok && tile < ntiles; tile += FWD_GROUPS * gridDim.x) {
        const int r0 = tile * MT;
        if (gt < MT) {
            const int r = r0 + gt;
            float f[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (r < n) {
                const float4 u = *reinterpret_cast<const float4*>(a.X + (size_t)r * RM_NX);
                const float4 w = *reinterpret_cast<const float4*>(a.X + (size_t)r * RM_NX + 4);
                f[0] = u.x; f[1] = u.y; f[2] = u.z; f[3] = u.w; f[4] = w.x; f[5] = w.y;
            }
            const uint4 lo = make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), 0u);
            const uint4 zz = make_uint4(0u, 0u, 0u, 0u);
            *reinterpret_cast<uint4*>(sX + tc::kmajor_off(gt, 0, KIN)) = lo;
            *reinterpret_cast<uint4*>(sX + tc::kmajor_off(gt, 8, KIN)) = zz;
            if (a.Hst && r < n) {
                uint4* d = reinterpret_cast<uint4*>(a.Hst + (size_t)r * KIN);
                d[0] = lo;
                d[1] = zz;
            }
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        grp_sync<FWD_GT>(1 + g);
        if (gt == 0) {
            tc::fence_after_sync();
            tc::mma_bf16(tbase, tc::sdesc(aX, 128, 256), tc::sdesc(aW + IW1, 128, 256), id128, 0);
            tc::mma_commit(gbar);
        }
        for (int l = 1; l <= 4; ++l) {
            ok = tc::mbar_wait(gbar, ph);
            ph ^= 1;
            ok = grp_sync_and<FWD_GT>(1 + g, ok);
            if (!ok) break;
            tc::fence_after_sync();
            const float* b = bias + (l - 1) * W;
            const int r = r0 + row;
#pragma unroll
            for (int c = 0; c < FWD_COLS / 16; ++c) {
                const int col = FWD_COLS * ch + 16 * c;
                float v[16], bb[16];
                tc::tmem_ld16(trow + (uint32_t)col, v);
#pragma unroll
                for (int i = 0; i < 16; i += 4) {
                    const float4 t4 = *reinterpret_cast<const float4*>(b + col + i);
                    bb[i] = t4.x; bb[i + 1] = t4.y; bb[i + 2] = t4.z; bb[i + 3] = t4.w;
                }
                uint32_t hb[8];
#pragma unroll
                for (int i = 0; i < 16; i += 2) {
                    const float z0 = v[i] + bb[i], z1 = v[i + 1] + bb[i + 1];
                    v[i] = z0;
                    v[i + 1] = z1;
                    hb[i >> 1] = pack_bf16(silu(z0), silu(z1));
                }
                const uint4 h0 = make_uint4(hb[0], hb[1], hb[2], hb[3]), h1 = make_uint4(hb[4], hb[5], hb[6], hb[7]);
                *reinterpret_cast<uint4*>(sH + tc::kmajor_off(row, col, W)) = h0;
                *reinterpret_cast<uint4*>(sH + tc::kmajor_off(row, col + 8, W)) = h1;
                if (a.Hst && r < n) {
                    uint4* d = reinterpret_cast<uint4*>(a.Hst + (size_t)n * KIN + (size_t)(l - 1) * n * W +
                                                        (size_t)r * W + col);
                    d[0] = h0;
                    d[1] = h1;
                }
                if (a.Zst && r < n) {
                    float4* d = reinterpret_cast<float4*>(a.Zst + (size_t)(l - 1) * n * W + (size_t)r * W + col);
#pragma unroll
                    for (int i = 0; i < 4; ++i) d[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
                }
            }
            tc::fence_async_smem();
            tc::fence_before_sync();
            grp_sync<FWD_GT>(1 + g);
            if (gt == 0) {
                tc::fence_after_sync();
                const bool last = l == 4;
                const uint32_t wl = last ? aW + IW5 : aW + IW2 + (uint32_t)(l - 1) * (W * W * 2);
                for (int kc = 0; kc < W / 16; ++kc)
                    tc::mma_bf16(last ? tout : tbase, tc::sdesc(aH + 256u * kc, 128, 2048),
                                 tc::sdesc(wl + 256u * kc, 128, 2048), last ? id16 : id128, kc > 0);
                tc::mma_commit(gbar);
            }
        }
        if (!ok) break;
        ok = tc::mbar_wait(gbar, ph);
        ph ^= 1;
        ok = grp_sync_and<FWD_GT>(1 + g, ok);
        if (!ok) break;
        tc::fence_after_sync();
        if (ch == 0) {
            float v[16];
            tc::tmem_ld16(tout + ((uint32_t)(32 * q) << 16), v);
            const int r = r0 + row;
            if (r < n) {
                const float* b5 = bias + 4 * W;
                *reinterpret_cast<float4*>(a.Y + (size_t)r * RM_NY) = make_float4(v[0] + b5[0], v[1] + b5[1], v[2] + b5[2], 0.f);
            }
        }
        tc::fence_before_sync();
        grp_sync<FWD_GT>(1 + g);
    }
    if (!ok && gt == 0 && a.err) atomicExch(a.err, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tall, 512);
}

// ---------------------------------------------------------------------------
// backward: dZ_{l-1} = (dZ_l W_l) * SiLU'(Z_{l-1})       (rows = samples)
//           dW_l    += dZ_l^T H_{l-1}, split over sample chunks (rows = outputs of layer l)
struct DhArgs {
    const float* dZ;      // n x ldz (FP32)
    int ldz, kl;          // kl: outputs of layer l padded to a multiple of 16
    const float* Wl;      // master W_l (out x 128)
    int outl;
    const float* Zp;      // Z_{l-1} (n x 128)
    float* dZp;           // out: dZ_{l-1} (n x 128)
    int n;
    int* err;
};

constexpr int DH_SA = 0, DH_SB = DH_SA + MT * W * 2, DH_BAR = DH_SB + W * W * 2, DH_SMEM = DH_BAR + 32;

__global__ void __launch_bounds__(256) km_mlp_dh(DhArgs a) {
    extern __shared__ __align__(128) uint8_t sm[];
    uint8_t* sA = sm + DH_SA;
    uint8_t* sB = sm + DH_SB;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + DH_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + DH_BAR + 16);
    const int ntiles = (a.n + MT - 1) / MT;
    if ((int)blockIdx.x >= ntiles) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int K = a.kl;
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tslot, 128);
        tc::tmem_relinquish();
    }
    // B operand (n = input i of layer l, k = output o): W_l[o][i]
    for (int e = tid; e < W * K; e += blockDim.x) {
        const int i = e / K, o = e - i * K;
        const float w = o < a.outl ? a.Wl[(size_t)o * W + i] : 0.f;
        *reinterpret_cast<__nv_bfloat16*>(sB + tc::kmajor_off(i, o, K)) = __float2bfloat16_rn(w);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot;
    const uint32_t aA = tc::smem_u32(sA), aB = tc::smem_u32(sB);
    const uint32_t idn = tc::idesc_bf16(MT, W);
    const int q = warp & 3, half = warp >> 2;
    const int row = 32 * q + lane;
    const uint32_t trow = tbase + ((uint32_t)(32 * q) << 16);
    uint32_t ph = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int r0 = tile * MT;
        // A operand (m = sample, k = output o of layer l): dZ_l, 8 columns per store
        for (int e = tid; e < MT * (K / 8); e += blockDim.x) {
            const int rr = e / (K / 8), k8 = (e - rr * (K / 8)) * 8;
            const int r = r0 + rr;
            float f[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (r < a.n) {
                const float4 u = *reinterpret_cast<const float4*>(a.dZ + (size_t)r * a.ldz + k8);
                const float4 w = *reinterpret_cast<const float4*>(a.dZ + (size_t)r * a.ldz + k8 + 4);
                f[0] = u.x; f[1] = u.y; f[2] = u.z; f[3] = u.w; f[4] = w.x; f[5] = w.y; f[6] = w.z; f[7] = w.w;
            }
            *reinterpret_cast<uint4*>(sA + tc::kmajor_off(rr, k8, K)) =
                make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t sbo = (uint32_t)(K / 8) * 128u;
            for (int kc = 0; kc < K / 16; ++kc)
                tc::mma_bf16(tbase, tc::sdesc(aA + 256u * kc, 128, sbo), tc::sdesc(aB + 256u * kc, 128, sbo), idn, kc > 0);
            tc::mma_commit(&bar[0]);
        }
        ok = tc::mbar_wait(&bar[0], ph);
        ph ^= 1;
        ok = __syncthreads_and(ok);
        if (!ok) break;
        tc::fence_after_sync();
        const int r = r0 + row;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int col = 64 * half + 16 * c;
            float v[16];
            tc::tmem_ld16(trow + (uint32_t)col, v);
            if (r < a.n) {
                const float* z = a.Zp + (size_t)r * W + col;
                float* d = a.dZp + (size_t)r * W + col;
#pragma unroll
                for (int i = 0; i < 16; i += 4) {
                    const float4 zz = *reinterpret_cast<const float4*>(z + i);
                    *reinterpret_cast<float4*>(d + i) =
                        make_float4(v[i] * dsilu(zz.x), v[i + 1] * dsilu(zz.y), v[i + 2] * dsilu(zz.z), v[i + 3] * dsilu(zz.w));
                }
            }
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    if (!ok && tid == 0 && a.err) atomicExch(a.err, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 128);
}

struct DwArgs {
    const float* dZ;             // n x ldz
    int ldz, outl;
    const __nv_bfloat16* Hp;     // H_{l-1}: n x nl (BF16)
    int nl;                      // 128, or 16 (layer 1, 6 inputs padded)
    int inl;                     // inputs of layer l actually stored in dW (6 or 128)
    float* dW;                   // out x inl, accumulated with atomics
    int n;
    int* err;
};

constexpr int DW_SA = 0, DW_SB = DW_SA + W * MT * 2, DW_BAR = DW_SB + W * MT * 2, DW_SMEM = DW_BAR + 32;

__global__ void __launch_bounds__(256) km_mlp_dw(DwArgs a) {
    extern __shared__ __align__(128) uint8_t sm[];
    uint8_t* sA = sm + DW_SA;
    uint8_t* sB = sm + DW_SB;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + DW_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + DW_BAR + 16);
    const int nchunk = (a.n + MT - 1) / MT;
    if ((int)blockIdx.x >= nchunk) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tslot, 128);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot;
    const uint32_t aA = tc::smem_u32(sA), aB = tc::smem_u32(sB);
    const uint32_t idn = tc::idesc_bf16(MT, a.nl);
    uint32_t ph = 0;
    bool ok = true;
    int first = 1;
    for (int ch = blockIdx.x; ch < nchunk; ch += gridDim.x) {
        const int b0 = ch * MT;
        // A (m = output o, k = sample b) and B (n = input i, k = sample b): pairs of samples per 4-byte store
        for (int e = tid; e < (MT / 2) * W; e += blockDim.x) {
            const int bp = e & (MT / 2 - 1), o = e >> 6;
            const int b = b0 + 2 * bp;
            float z0 = 0.f, z1 = 0.f;
            if (o < a.outl) {
                if (b < a.n) z0 = a.dZ[(size_t)b * a.ldz + o];
                if (b + 1 < a.n) z1 = a.dZ[(size_t)(b + 1) * a.ldz + o];
            }
            *reinterpret_cast<uint32_t*>(sA + tc::kmajor_off(o, 2 * bp, MT)) = pack_bf16(z0, z1);
        }
        for (int e = tid; e < (MT / 2) * a.nl; e += blockDim.x) {
            const int bp = e & (MT / 2 - 1), i = e >> 6;
            const int b = b0 + 2 * bp;
            __nv_bfloat16 h0 = __float2bfloat16_rn(0.f), h1 = h0;
            if (b < a.n) h0 = a.Hp[(size_t)b * a.nl + i];
            if (b + 1 < a.n) h1 = a.Hp[(size_t)(b + 1) * a.nl + i];
            __nv_bfloat162 hh;
            hh.x = h0;
            hh.y = h1;
            *reinterpret_cast<__nv_bfloat162*>(sB + tc::kmajor_off(i, 2 * bp, MT)) = hh;
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            for (int kc = 0; kc < MT / 16; ++kc) {
                tc::mma_bf16(tbase, tc::sdesc(aA + 256u * kc, 128, 2048), tc::sdesc(aB + 256u * kc, 128, 2048), idn,
                             (kc > 0 || !first) ? 1u : 0u);
            }
            tc::mma_commit(&bar[0]);
        }
        first = 0;
        ok = tc::mbar_wait(&bar[0], ph);       // the operands are rewritten by the next chunk
        ph ^= 1;
        ok = __syncthreads_and(ok);
        if (!ok) break;
    }
    if (ok) {
        tc::fence_after_sync();
        const int q = warp & 3, half = warp >> 2;
        const int o = 32 * q + lane;
        const uint32_t trow = tbase + ((uint32_t)(32 * q) << 16);
        // the two column halves of the accumulator go to the two warps of a lane quarter
        const int nblk = a.nl / 16, per = (nblk + 1) / 2;
        const int c0 = half * per, c1 = min(nblk, c0 + per);
        for (int c = c0; c < c1; ++c) {
            float v[16];
            tc::tmem_ld16(trow + (uint32_t)(16 * c), v);
            if (o < a.outl) {
                for (int i = 0; i < 16; ++i) {
                    const int col = 16 * c + i;
                    if (col < a.inl) atomicAdd(&a.dW[(size_t)o * a.inl + col], v[i]);
                }
            }
        }
    }
    if (!ok && tid == 0 && a.err) atomicExch(a.err, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 128);
}

// ---------------------------------------------------------------------------
// elementwise parts of a training iteration

// dZ_5 = 2 (Y - T) / (3 n) in a n x 16 buffer (columns 3.. zero); loss += sum (Y - T)^2 / (3 n)
__global__ void km_mlp_loss(const float* Y, const float* T, int n, float* dZ5, double* loss) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (r < n) {
        const float sc = 2.f / (3.f * (float)n);
        float d[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) d[j] = 0.f;
#pragma unroll
        for (int j = 0; j < NOUT; ++j) {
            const float e = Y[(size_t)r * RM_NY + j] - T[(size_t)r * RM_NY + j];
            d[j] = sc * e;
            l += (double)e * (double)e;
        }
        float4* o = reinterpret_cast<float4*>(dZ5 + (size_t)r * NO);
#pragma unroll
        for (int j = 0; j < 4; ++j) o[j] = make_float4(d[4 * j], d[4 * j + 1], d[4 * j + 2], d[4 * j + 3]);
    }
    // block sum, one atomic per block
    __shared__ double s[256];
    s[threadIdx.x] = l;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, s[0] / (3.0 * (double)n));
}

// db[o] += sum over rows of dZ[r][o], o < nout
__global__ void km_mlp_colsum(const float* dZ, int ldz, int nout, int n, float* db) {
    const int o = threadIdx.x;
    const int r0 = blockIdx.x * 256;
    if (o >= nout) return;
    float s = 0.f;
    for (int r = r0; r < min(n, r0 + 256); ++r) s += dZ[(size_t)r * ldz + o];
    atomicAdd(&db[o], s);
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8) with the step count kept on the device; zeroes the gradient
__global__ void km_mlp_adam(float* P, float* G, float* M, float* V, int np, float lr, int* tstep) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = *tstep + 1;
    if (i < np) {
        const float g = G[i];
        const float m = 0.9f * M[i] + 0.1f * g;
        const float v = 0.999f * V[i] + 0.001f * g * g;
        M[i] = m;
        V[i] = v;
        const float mh = m / (1.f - powf(0.9f, (float)t)), vh = v / (1.f - powf(0.999f, (float)t));
        P[i] -= lr * mh / (sqrtf(vh) + 1e-8f);
        G[i] = 0.f;
    }
}

__global__ void km_mlp_tick(int* tstep) { *tstep += 1; }

// FP32 master parameters -> BF16 K-major image + FP32 biases
__global__ void km_mlp_pack(const float* P, uint8_t* img) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    // W1: 128 x 16 (inputs 6..15 zero)
    if (e < W * KIN) {
        const int o = e / KIN, i = e - o * KIN;
        const float w = i < NIN ? P[OW1 + o * NIN + i] : 0.f;
        *reinterpret_cast<__nv_bfloat16*>(img + IW1 + tc::kmajor_off(o, i, KIN)) = __float2bfloat16_rn(w);
    }
    // W2..W4
    if (e < 3 * W * W) {
        const int l = e / (W * W), r = e - l * W * W;
        const int o = r / W, i = r - o * W;
        const float w = P[w_off(l + 2) + o * W + i];
        *reinterpret_cast<__nv_bfloat16*>(img + IW2 + l * (W * W * 2) + tc::kmajor_off(o, i, W)) = __float2bfloat16_rn(w);
    }
    // W5: 16 x 128 (outputs 3..15 zero)
    if (e < NO * W) {
        const int o = e / W, i = e - o * W;
        const float w = o < NOUT ? P[OW5 + o * W + i] : 0.f;
        *reinterpret_cast<__nv_bfloat16*>(img + IW5 + tc::kmajor_off(o, i, W)) = __float2bfloat16_rn(w);
    }
    if (e < 4 * W + NO) {
        float b;
        if (e < 4 * W) b = P[b_off(e / W + 1) + (e % W)];
        else b = (e - 4 * W) < NOUT ? P[OB5 + (e - 4 * W)] : 0.f;
        reinterpret_cast<float*>(img + IBIAS)[e] = b;
    }
}

// mean of the 3 used target columns over the data set (rows: *ndev clamped to N, or N)
__global__ void km_mlp_tmean(const float* __restrict__ T, long long N, const long long* ndev, double* acc) {
    const long long n = ndev ? min(*ndev, N) : N;
    double s[NOUT] = {};
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x)
#pragma unroll
        for (int k = 0; k < NOUT; ++k) s[k] += (double)T[(size_t)r * RM_NY + k];
#pragma unroll
    for (int k = 0; k < NOUT; ++k) {
        double v = s[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&acc[k], v);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&acc[NOUT], (double)n);
}

__global__ void km_mlp_setbias(float* P, const double* acc) {
    const int k = threadIdx.x;
    if (k < NOUT && acc[NOUT] > 0.0) P[OB5 + k] = (float)(acc[k] / acc[NOUT]);
}

// random mini-batch: rows idx = hash(seed, step, r) mod N of the data set
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__global__ void km_mlp_gather(const float* DX, const float* DT, long long N, const long long* ndev, int n,
                              uint64_t seed, const int* tstep, float* X, float* T) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    long long Nn = ndev ? min(*ndev, N) : N;
    if (Nn <= 0) Nn = 1;
    const uint64_t h = mix64(seed ^ mix64(((uint64_t)(*tstep) << 32) ^ (uint64_t)r));
    const long long k = (long long)(h % (uint64_t)Nn);
    const float4* sx = reinterpret_cast<const float4*>(DX + (size_t)k * RM_NX);
    float4* dx = reinterpret_cast<float4*>(X + (size_t)r * RM_NX);
    dx[0] = sx[0];
    dx[1] = sx[1];
    *reinterpret_cast<float4*>(T + (size_t)r * RM_NY) = *reinterpret_cast<const float4*>(DT + (size_t)k * RM_NY);
}

// failure detection: a wait on an mbarrier that nothing arrives at gives up after `ns`
__global__ void km_wait_selftest(uint64_t ns, int* out) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::mbar_fence_init();
    }
    __syncthreads();
    const bool ok = tc::mbar_wait(&bar, 0, ns);
    if (threadIdx.x == 0) out[0] = ok ? 0 : 1;
}

}  // namespace mlp

// ---------------------------------------------------------------------------
// host side of the network object
using namespace mlp;

struct MlpDev {
    float* P = nullptr;        // master parameters
    float* G = nullptr;        // gradient
    float* M = nullptr;        // Adam moments
    float* V = nullptr;
    uint8_t* img = nullptr;    // packed forward image
    int* tstep = nullptr;      // Adam step count
    int* err = nullptr;
    double* loss = nullptr;
    // training scratch for a batch of `bcap` rows
    int bcap = 0;
    float *X = nullptr, *T = nullptr, *Y = nullptr, *Z = nullptr, *dZa = nullptr, *dZb = nullptr, *dZ5 = nullptr;
    __nv_bfloat16* H = nullptr;
    // recorded (features, exact label) pairs
    long long rcap = 0;
    float *RX = nullptr, *RT = nullptr;
    long long* rcount = nullptr;
};

}  // namespace ep

struct ep_mlp {
    ep::MlpDev d;
    cudaStream_t s = nullptr;
    double l2g = 0.0;                 // lambda / (2G) of the material the labels use
    std::string err;
    cudaGraphExec_t train_graph = nullptr;
    int graph_batch = 0;
    float graph_lr = 0.f;
    uint64_t graph_seed = 0;
    const float* graph_dx = nullptr;
    long long graph_n = 0;
    int sms = 0;
    bool fresh = true;                // initial weights: the first training call sets the output bias
};

namespace ep {

static void mlp_fwd_launch(ep_mlp* m, const float* X, int n, const int* ndev, float* Y, bool train, cudaStream_t s) {
    FwdArgs a;
    a.X = X;
    a.n = n;
    a.ndev = ndev;
    a.Y = Y;
    a.img = m->d.img;
    a.Hst = train ? m->d.H : nullptr;
    a.Zst = train ? m->d.Z : nullptr;
    a.err = m->d.err;
    const int tiles = (n + MT - 1) / MT;
    const int grid = ndev ? m->sms : std::max(1, std::min((tiles + FWD_GROUPS - 1) / FWD_GROUPS, m->sms));
    km_mlp_fwd<<<grid, FWD_THREADS, FWD_SMEM, s>>>(a);
}

void mlp_infer(ep_mlp* m, const float* X, const int* ndev, int cap, float* Y, cudaStream_t s) {
    mlp_fwd_launch(m, X, cap, ndev, Y, false, s);
}

const uint8_t* mlp_image(ep_mlp* m) { return m->d.img; }
float* mlp_record_x(ep_mlp* m) { return m->d.RX; }
float* mlp_record_t(ep_mlp* m) { return m->d.RT; }
long long* mlp_record_count(ep_mlp* m) { return m->d.rcount; }
long long mlp_record_cap(ep_mlp* m) { return m->d.rcap; }
int* mlp_err(ep_mlp* m) { return m->d.err; }

// one forward + backward over a batch already in d.X / d.T (n rows, n <= bcap); gradient into d.G
static void mlp_fwd_bwd(ep_mlp* m, int n, cudaStream_t s) {
    MlpDev& d = m->d;
    mlp_fwd_launch(m, d.X, n, nullptr, d.Y, true, s);
    km_mlp_loss<<<(n + 255) / 256, 256, 0, s>>>(d.Y, d.T, n, d.dZ5, d.loss);
    const int tiles = (n + MT - 1) / MT;
    const int gdh = std::max(1, std::min(tiles, 3 * m->sms));
    const int gdw = std::max(1, std::min(tiles, 2 * m->sms));
    const float* dZ = d.dZ5;
    int ldz = NO;
    for (int l = 5; l >= 1; --l) {
        // dW_l, db_l
        DwArgs w;
        w.dZ = dZ;
        w.ldz = ldz;
        w.outl = n_out(l);
        w.nl = l == 1 ? KIN : W;
        w.inl = n_in(l);
        w.Hp = l == 1 ? d.H : d.H + (size_t)n * KIN + (size_t)(l - 2) * n * W;
        w.dW = d.G + w_off(l);
        w.n = n;
        w.err = d.err;
        km_mlp_dw<<<gdw, 256, DW_SMEM, s>>>(w);
        km_mlp_colsum<<<(n + 255) / 256, 128, 0, s>>>(dZ, ldz, n_out(l), n, d.G + b_off(l));
        if (l == 1) break;
        // dZ_{l-1}
        DhArgs h;
        h.dZ = dZ;
        h.ldz = ldz;
        h.kl = l == 5 ? NO : W;
        h.Wl = d.P + w_off(l);
        h.outl = n_out(l);
        h.Zp = d.Z + (size_t)(l - 2) * n * W;
        float* out = (dZ == d.dZa) ? d.dZb : d.dZa;
        h.dZp = out;
        h.n = n;
        h.err = d.err;
        km_mlp_dh<<<gdh, 256, DH_SMEM, s>>>(h);
        dZ = out;
        ldz = W;
    }
}

static cudaError_t mlp_set_attrs() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(km_mlp_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, FWD_SMEM);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(km_mlp_dh, cudaFuncAttributeMaxDynamicSharedMemorySize, DH_SMEM);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(km_mlp_dw, cudaFuncAttributeMaxDynamicSharedMemorySize, DW_SMEM);
    if (e == cudaSuccess) done = true;
    return e;
}

cudaError_t mlp_prepare() { return mlp_set_attrs(); }

}  // namespace ep

using namespace ep;

static ep_status mfail(ep_mlp* m, ep_status st, const std::string& msg) {
    if (m) m->err = msg;
    else set_global_error(msg.c_str());
    return st;
}
static ep_status mcuda(ep_mlp* m, cudaError_t e, const char* where) {
    std::string msg = std::string(where) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return mfail(m, EP_ERR_CUDA, msg);
}
#define MCK(m, call)                                              \
    do {                                                          \
        cudaError_t e__ = (call);                                 \
        if (e__ != cudaSuccess) return mcuda((m), e__, #call);    \
    } while (0)

static ep_status mlp_check_err(ep_mlp* m) {
    int e = 0;
    MCK(m, cudaMemcpyAsync(&e, m->d.err, sizeof(int), cudaMemcpyDeviceToHost, m->s));
    MCK(m, cudaStreamSynchronize(m->s));
    if (e) return mfail(m, EP_ERR_TIMEOUT, "tensor-core wait timed out in an MLP kernel");
    return EP_OK;
}

static ep_status ensure_batch(ep_mlp* m, int n) {
    MlpDev& d = m->d;
    if (n <= d.bcap) return EP_OK;
    if (m->train_graph) {                    // it points at the buffers about to be replaced
        cudaGraphExecDestroy(m->train_graph);
        m->train_graph = nullptr;
    }
    cudaFree(d.X); cudaFree(d.T); cudaFree(d.Y); cudaFree(d.Z); cudaFree(d.dZa); cudaFree(d.dZb); cudaFree(d.dZ5);
    cudaFree(d.H);
    d.X = d.T = d.Y = d.Z = d.dZa = d.dZb = d.dZ5 = nullptr;
    d.H = nullptr;
    d.bcap = 0;
    const size_t N = (size_t)((n + MT - 1) / MT) * MT;
    MCK(m, cudaMalloc(&d.X, N * RM_NX * sizeof(float)));
    MCK(m, cudaMalloc(&d.T, N * RM_NY * sizeof(float)));
    MCK(m, cudaMalloc(&d.Y, N * RM_NY * sizeof(float)));
    MCK(m, cudaMalloc(&d.Z, 4 * N * W * sizeof(float)));
    MCK(m, cudaMalloc(&d.dZa, N * W * sizeof(float)));
    MCK(m, cudaMalloc(&d.dZb, N * W * sizeof(float)));
    MCK(m, cudaMalloc(&d.dZ5, N * NO * sizeof(float)));
    MCK(m, cudaMalloc(&d.H, (N * KIN + 4 * N * W) * sizeof(__nv_bfloat16)));
    d.bcap = (int)N;
    return EP_OK;
}

// He-style initial weights from a seeded splitmix64 / Box-Muller stream (host)
static void init_params(std::vector<float>& P, uint64_t seed) {
    uint64_t st = seed ^ 0x2545f4914f6cdd1dull;
    auto next = [&]() {
        st += 0x9e3779b97f4a7c15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    };
    auto unif = [&]() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
    P.assign(NPARAM, 0.f);
    for (int l = 1; l <= 5; ++l) {
        const int ni = n_in(l), no = n_out(l);
        // He initialisation; the output layer starts 10x smaller (its bias starts at the mean target)
        const double sd = l == 5 ? 0.1 * std::sqrt(1.0 / ni) : std::sqrt(2.0 / ni);
        for (int k = 0; k < ni * no; ++k) {
            const double u1 = unif(), u2 = unif();
            P[w_off(l) + k] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
}

extern "C" {

ep_status epgpu_mlp_create(uint64_t seed, double lambda_over_2G, ep_mlp** out) {
    if (!out) return EP_ERR_ARG;
    *out = nullptr;
    ep_mlp* m = new ep_mlp();
    m->l2g = lambda_over_2G;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = mlp_prepare();
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->s, cudaStreamNonBlocking);
    MlpDev& d = m->d;
    auto al = [&](auto** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc((void**)p, bytes);
        if (e == cudaSuccess) e = cudaMemset(*p, 0, bytes);
    };
    al(&d.P, NPARAM * sizeof(float));
    al(&d.G, NPARAM * sizeof(float));
    al(&d.M, NPARAM * sizeof(float));
    al(&d.V, NPARAM * sizeof(float));
    al(&d.img, IMG_BYTES);
    al(&d.tstep, sizeof(int));
    al(&d.err, sizeof(int));
    al(&d.loss, sizeof(double));
    al(&d.rcount, sizeof(long long));
    if (e != cudaSuccess) {
        std::string msg = std::string("mlp create: ") + cudaGetErrorString(e);
        cudaGetLastError();
        epgpu_mlp_destroy(m);
        return mfail(nullptr, EP_ERR_CUDA, msg);
    }
    std::vector<float> P;
    init_params(P, seed);
    ep_status st = epgpu_mlp_set_params(m, P.data(), NPARAM);
    if (st != EP_OK) {
        epgpu_mlp_destroy(m);
        return st;
    }
    m->fresh = true;
    *out = m;
    return EP_OK;
}

ep_status epgpu_mlp_destroy(ep_mlp* m) {
    if (!m) return EP_OK;
    MlpDev& d = m->d;
    if (m->s) cudaStreamSynchronize(m->s);
    if (m->train_graph) cudaGraphExecDestroy(m->train_graph);
    void* ps[] = {d.P, d.G, d.M, d.V, d.img, d.tstep, d.err, d.loss, d.X, d.T, d.Y, d.Z, d.dZa, d.dZb, d.dZ5, d.H,
                  d.RX, d.RT, d.rcount};
    for (void* p : ps)
        if (p) cudaFree(p);
    if (m->s) cudaStreamDestroy(m->s);
    delete m;
    return EP_OK;
}

const char* epgpu_mlp_last_error(ep_mlp* m) { return m ? m->err.c_str() : ""; }

ep_status epgpu_mlp_set_params(ep_mlp* m, const float* p, int64_t n) {
    if (!m || !p || n != NPARAM) return EP_ERR_ARG;
    MCK(m, cudaMemcpyAsync(m->d.P, p, NPARAM * sizeof(float), cudaMemcpyHostToDevice, m->s));
    MCK(m, cudaMemsetAsync(m->d.M, 0, NPARAM * sizeof(float), m->s));
    MCK(m, cudaMemsetAsync(m->d.V, 0, NPARAM * sizeof(float), m->s));
    MCK(m, cudaMemsetAsync(m->d.G, 0, NPARAM * sizeof(float), m->s));
    MCK(m, cudaMemsetAsync(m->d.tstep, 0, sizeof(int), m->s));
    km_mlp_pack<<<(3 * W * W + 255) / 256, 256, 0, m->s>>>(m->d.P, m->d.img);
    MCK(m, cudaGetLastError());
    MCK(m, cudaStreamSynchronize(m->s));
    m->fresh = false;
    return EP_OK;
}

ep_status epgpu_mlp_get_params(ep_mlp* m, float* p, int64_t n) {
    if (!m || !p || n != NPARAM) return EP_ERR_ARG;
    MCK(m, cudaMemcpyAsync(p, m->d.P, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, m->s));
    MCK(m, cudaStreamSynchronize(m->s));
    return EP_OK;
}

ep_status epgpu_mlp_forward(ep_mlp* m, const float* x, int64_t n, float* y) {
    if (!m || (n > 0 && (!x || !y)) || n < 0 || n > (1 << 30)) return EP_ERR_ARG;
    if (n == 0) return EP_OK;
    ep_status st;
    if ((st = ensure_batch(m, (int)n)) != EP_OK) return st;
    MlpDev& d = m->d;
    MCK(m, cudaMemcpyAsync(d.X, x, (size_t)n * RM_NX * sizeof(float), cudaMemcpyHostToDevice, m->s));
    mlp_fwd_launch(m, d.X, (int)n, nullptr, d.Y, false, m->s);
    MCK(m, cudaGetLastError());
    MCK(m, cudaMemcpyAsync(y, d.Y, (size_t)n * RM_NY * sizeof(float), cudaMemcpyDeviceToHost, m->s));
    return mlp_check_err(m);
}

ep_status epgpu_mlp_time(ep_mlp* m, int64_t n, int32_t reps, double* ms_per_launch) {
    if (!m || !ms_per_launch || n <= 0 || n > (1 << 30) || reps <= 0) return EP_ERR_ARG;
    ep_status st;
    if ((st = ensure_batch(m, (int)n)) != EP_OK) return st;
    MlpDev& d = m->d;
    MCK(m, cudaMemsetAsync(d.X, 0, (size_t)n * RM_NX * sizeof(float), m->s));
    mlp_fwd_launch(m, d.X, (int)n, nullptr, d.Y, false, m->s);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    MCK(m, cudaEventCreate(&e0));
    cudaError_t e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaEventRecord(e0, m->s);
    for (int i = 0; i < reps && e == cudaSuccess; ++i) {
        mlp_fwd_launch(m, d.X, (int)n, nullptr, d.Y, false, m->s);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, m->s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    MCK(m, e);
    if ((st = mlp_check_err(m)) != EP_OK) return st;
    *ms_per_launch = (double)ms / reps;
    return EP_OK;
}

ep_status epgpu_mlp_grad(ep_mlp* m, const float* x, const float* t, int64_t n, float* grad, double* loss) {
    if (!m || !x || !t || !grad || n <= 0 || n > (1 << 26)) return EP_ERR_ARG;
    ep_status st;
    if ((st = ensure_batch(m, (int)n)) != EP_OK) return st;
    MlpDev& d = m->d;
    MCK(m, cudaMemcpyAsync(d.X, x, (size_t)n * RM_NX * sizeof(float), cudaMemcpyHostToDevice, m->s));
    MCK(m, cudaMemcpyAsync(d.T, t, (size_t)n * RM_NY * sizeof(float), cudaMemcpyHostToDevice, m->s));
    MCK(m, cudaMemsetAsync(d.G, 0, NPARAM * sizeof(float), m->s));
    MCK(m, cudaMemsetAsync(d.loss, 0, sizeof(double), m->s));
    mlp_fwd_bwd(m, (int)n, m->s);
    MCK(m, cudaGetLastError());
    MCK(m, cudaMemcpyAsync(grad, d.G, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, m->s));
    double l = 0.0;
    MCK(m, cudaMemcpyAsync(&l, d.loss, sizeof(double), cudaMemcpyDeviceToHost, m->s));
    if ((st = mlp_check_err(m)) != EP_OK) return st;
    MCK(m, cudaMemsetAsync(d.G, 0, NPARAM * sizeof(float), m->s));
    if (loss) *loss = l;
    return EP_OK;
}

// `iters` Adam steps on random mini-batches of `batch` rows drawn from n data rows
// (x: n x 8, t: n x 4; host memory, or the recorded pairs when x == NULL)
ep_status epgpu_mlp_train(ep_mlp* m, const float* x, const float* t, int64_t n, int32_t iters, int32_t batch,
                          float lr, uint64_t seed, double* loss_out) {
    if (!m || iters < 0 || batch <= 0 || batch > (1 << 20) || !(lr > 0.f)) return EP_ERR_ARG;
    MlpDev& d = m->d;
    const float* DX;
    const float* DT;
    const long long* ndev = nullptr;
    std::vector<float*> tmp;
    long long N;
    if (x) {
        if (!t || n <= 0) return EP_ERR_ARG;
        float *a = nullptr, *b = nullptr;
        MCK(m, cudaMalloc(&a, (size_t)n * RM_NX * sizeof(float)));
        tmp.push_back(a);
        MCK(m, cudaMalloc(&b, (size_t)n * RM_NY * sizeof(float)));
        tmp.push_back(b);
        MCK(m, cudaMemcpyAsync(a, x, (size_t)n * RM_NX * sizeof(float), cudaMemcpyHostToDevice, m->s));
        MCK(m, cudaMemcpyAsync(b, t, (size_t)n * RM_NY * sizeof(float), cudaMemcpyHostToDevice, m->s));
        DX = a;
        DT = b;
        N = n;
    } else {
        if (!d.RX) return mfail(m, EP_ERR_STATE, "no record buffer (epgpu_mlp_record_buffer)");
        long long c = 0;
        MCK(m, cudaDeviceSynchronize());
        MCK(m, cudaMemcpy(&c, d.rcount, sizeof(long long), cudaMemcpyDeviceToHost));
        if (c <= 0) return mfail(m, EP_ERR_STATE, "the record buffer is empty (run the step with EP_RMAP_RECORD)");
        DX = d.RX;
        DT = d.RT;
        N = d.rcap;
        ndev = d.rcount;
    }
    ep_status st;
    if ((st = ensure_batch(m, batch)) != EP_OK) return st;
    if (m->fresh) {
        // first training of the initial weights: the output bias starts at the mean target
        double* acc = nullptr;
        MCK(m, cudaMalloc(&acc, (NOUT + 1) * sizeof(double)));
        tmp.push_back(reinterpret_cast<float*>(acc));
        MCK(m, cudaMemsetAsync(acc, 0, (NOUT + 1) * sizeof(double), m->s));
        km_mlp_tmean<<<m->sms, 256, 0, m->s>>>(DT, N, ndev, acc);
        km_mlp_setbias<<<1, 32, 0, m->s>>>(d.P, acc);
        km_mlp_pack<<<(3 * W * W + 255) / 256, 256, 0, m->s>>>(d.P, d.img);
        MCK(m, cudaGetLastError());
        m->fresh = false;
    }
    MCK(m, cudaMemsetAsync(d.loss, 0, sizeof(double), m->s));
    // one iteration = gather, forward, backward, Adam, repack; captured once per (data, batch, lr, seed)
    if (!m->train_graph || m->graph_batch != batch || m->graph_lr != lr || m->graph_seed != seed ||
        m->graph_dx != DX || m->graph_n != N) {
        if (m->train_graph) cudaGraphExecDestroy(m->train_graph);
        m->train_graph = nullptr;
        cudaGraph_t g;
        MCK(m, cudaStreamBeginCapture(m->s, cudaStreamCaptureModeThreadLocal));
        km_mlp_gather<<<(batch + 255) / 256, 256, 0, m->s>>>(DX, DT, N, ndev, batch, seed, d.tstep, d.X, d.T);
        mlp_fwd_bwd(m, batch, m->s);
        km_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, m->s>>>(d.P, d.G, d.M, d.V, NPARAM, lr, d.tstep);
        km_mlp_tick<<<1, 1, 0, m->s>>>(d.tstep);
        km_mlp_pack<<<(3 * W * W + 255) / 256, 256, 0, m->s>>>(d.P, d.img);
        cudaError_t e = cudaStreamEndCapture(m->s, &g);
        if (e != cudaSuccess) return mcuda(m, e, "training graph capture");
        e = cudaGraphInstantiate(&m->train_graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return mcuda(m, e, "training graph instantiate");
        m->graph_batch = batch;
        m->graph_lr = lr;
        m->graph_seed = seed;
        m->graph_dx = DX;
        m->graph_n = N;
    }
    for (int it = 0; it < iters; ++it) {
        if (it == iters - 1) MCK(m, cudaMemsetAsync(d.loss, 0, sizeof(double), m->s));
        MCK(m, cudaGraphLaunch(m->train_graph, m->s));
    }
    double l = 0.0;
    MCK(m, cudaMemcpyAsync(&l, d.loss, sizeof(double), cudaMemcpyDeviceToHost, m->s));
    st = mlp_check_err(m);
    for (float* p : tmp) cudaFree(p);
    if (tmp.size()) m->graph_dx = nullptr;   // the temporary data set is gone: recapture next time
    if (tmp.size() && m->train_graph) {
        cudaGraphExecDestroy(m->train_graph);
        m->train_graph = nullptr;
    }
    if (loss_out) *loss_out = l;
    return st;
}

ep_status epgpu_selftest_wait_timeout(int64_t timeout_ns) {
    if (timeout_ns <= 0 || timeout_ns > 2000000000LL) return EP_ERR_ARG;
    int* d = nullptr;
    int r = -1;
    cudaError_t e = cudaMalloc(&d, sizeof(int));
    if (e == cudaSuccess) {
        km_wait_selftest<<<1, 32>>>((uint64_t)timeout_ns, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&r, d, sizeof(int), cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (e != cudaSuccess) return mcuda(nullptr, e, "wait self test");
    return r == 1 ? EP_ERR_TIMEOUT : EP_OK;
}

ep_status epgpu_mlp_label(const float* x, int64_t n, double lambda_over_2G, float* y) {
    if ((n > 0 && (!x || !y)) || n < 0) return EP_ERR_ARG;
    for (int64_t r = 0; r < n; ++r) rm_label(x + r * RM_NX, lambda_over_2G, y + r * RM_NY);
    return EP_OK;
}

ep_status epgpu_mlp_record_buffer(ep_mlp* m, int64_t capacity) {
    if (!m || capacity < 0) return EP_ERR_ARG;
    MlpDev& d = m->d;
    if (capacity != d.rcap) {
        if (d.RX) cudaFree(d.RX);
        if (d.RT) cudaFree(d.RT);
        d.RX = d.RT = nullptr;
        d.rcap = 0;
        if (capacity > 0) {
            MCK(m, cudaMalloc(&d.RX, (size_t)capacity * RM_NX * sizeof(float)));
            MCK(m, cudaMalloc(&d.RT, (size_t)capacity * RM_NY * sizeof(float)));
        }
        d.rcap = capacity;
    }
    MCK(m, cudaMemsetAsync(d.rcount, 0, sizeof(long long), m->s));
    MCK(m, cudaStreamSynchronize(m->s));
    return EP_OK;
}

ep_status epgpu_mlp_recorded(ep_mlp* m, int64_t* count, float* x, float* t, int64_t cap) {
    if (!m || !count) return EP_ERR_ARG;
    long long c = 0;
    MCK(m, cudaDeviceSynchronize());
    MCK(m, cudaMemcpy(&c, m->d.rcount, sizeof(long long), cudaMemcpyDeviceToHost));
    *count = c;
    const long long k = std::min<long long>(std::min<long long>(c, m->d.rcap), cap);
    if (k > 0 && x) MCK(m, cudaMemcpy(x, m->d.RX, (size_t)k * RM_NX * sizeof(float), cudaMemcpyDeviceToHost));
    if (k > 0 && t) MCK(m, cudaMemcpy(t, m->d.RT, (size_t)k * RM_NY * sizeof(float), cudaMemcpyDeviceToHost));
    return EP_OK;
}

}  // extern "C"
