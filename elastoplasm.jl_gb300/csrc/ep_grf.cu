// ep_grf.cu -- seeded Gaussian random fields at the material points (cohesion
// fields of the scaled-up slumps).
//
// The reference draws its cohesion field with a harmonic sum on a regular grid
// (utils/setup/mpts/GRF.jl:66-141, Gaussian covariance); its exponential branch
// is not wired in (mpts_populate.jl:49-51).  This generator is written from the
// published randomization (spectral) method for stationary Gaussian fields
// (Shinozuka & Deodatis 1991; Kramer, Kurbanmuradov & Sabelfeld 2007):
//
//   f(x) = sigma / sqrt(Nh) * sum_k [ xi_k cos(kappa_k . x) + eta_k sin(kappa_k . x) ]
//
// with xi_k, eta_k ~ N(0, 1) and the wave vectors kappa_k drawn from the
// spectral density of the correlation function rho(|dx / ell|):
//   exponential rho(r) = exp(-r): radial CDF 1 - (1 + k^2)^(-1/2) in 2d,
//       (2 / pi)(atan k - k / (1 + k^2)) in 3d, uniform direction;
//   Gaussian rho(r) = exp(-r^2): each component ~ N(0, 2);
// each component then divided by its correlation length ell_i.  The field is
// evaluated directly at the point positions; the value is mean + f, clamped
// from below at vmin.
//
// Random numbers: one splitmix64 stream from the seed, 8 uniforms per harmonic
// in (0, 1): u0, u1, u2 wave vector, u4, u5 amplitudes (Box-Muller).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/epgpu.h"
#include "ep_internal.h"

namespace ep {
namespace {

struct SplitMix {
    uint64_t s;
    uint64_t next() {
        s += 0x9e3779b97f4a7c15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double unif() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
};

constexpr double TWO_PI = 6.283185307179586476925286766559;

// inverse of the 3d exponential radial CDF by bisection on k
double inv_exp3(double u) {
    auto F = [](double k) { return (2.0 / 3.14159265358979323846) * (std::atan(k) - k / (1.0 + k * k)); };
    double lo = 0.0, hi = 1.0;
    while (F(hi) < u && hi < 1e300) hi *= 2.0;
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (F(mid) < u) lo = mid;
        else hi = mid;
        if (hi - lo <= 1e-15 * hi) break;
    }
    return 0.5 * (lo + hi);
}

}  // namespace

// harmonics: kappa (nh x dim, row-major), amplitudes ab (nh x 2)
void grf_spectrum(const ep_grf& g, double* kappa, double* ab) {
    SplitMix r{g.seed};
    const int d = g.dim;
    for (int k = 0; k < g.nh; ++k) {
        double u[8];
        for (int i = 0; i < 8; ++i) u[i] = r.unif();
        double kv[3] = {0.0, 0.0, 0.0};
        if (g.covariance == EP_GRF_EXPONENTIAL) {
            double kr;
            if (d == 2) {
                const double q = 1.0 / (1.0 - u[0]);
                kr = std::sqrt(q * q - 1.0);
                const double th = TWO_PI * u[1];
                kv[0] = kr * std::cos(th);
                kv[1] = kr * std::sin(th);
            } else {
                kr = inv_exp3(u[0]);
                const double ct = 1.0 - 2.0 * u[1], st = std::sqrt(std::max(0.0, 1.0 - ct * ct));
                const double ph = TWO_PI * u[2];
                kv[0] = kr * st * std::cos(ph);
                kv[1] = kr * st * std::sin(ph);
                kv[2] = kr * ct;
            }
        } else {
            // N(0, 2) per component: Box-Muller on (u0, u1) and (u2, u3)
            const double r1 = std::sqrt(-2.0 * std::log(u[0])), r2 = std::sqrt(-2.0 * std::log(u[2]));
            kv[0] = std::sqrt(2.0) * r1 * std::cos(TWO_PI * u[1]);
            kv[1] = std::sqrt(2.0) * r1 * std::sin(TWO_PI * u[1]);
            kv[2] = std::sqrt(2.0) * r2 * std::cos(TWO_PI * u[3]);
        }
        for (int i = 0; i < d; ++i) kappa[(size_t)k * d + i] = kv[i] / g.ell[i];
        const double ra = std::sqrt(-2.0 * std::log(u[4]));
        ab[2 * (size_t)k] = ra * std::cos(TWO_PI * u[5]);
        ab[2 * (size_t)k + 1] = ra * std::sin(TWO_PI * u[5]);
    }
}

constexpr int GRF_CHUNK = 512;

// one thread per point; harmonics staged through shared memory; the phase is
// formed and reduced to [-pi, pi] in FP64, the sine and cosine in FP32, the
// chunk sums in FP32 and the total in FP64
template <int D>
__global__ void __launch_bounds__(256) k_grf(const double* __restrict__ kappa, const float* __restrict__ ab, int nh,
                                             const double* __restrict__ x, long long np, double scale, double mean,
                                             double vmin, double* __restrict__ out) {
    __shared__ double sk[GRF_CHUNK * D];
    __shared__ float sab[GRF_CHUNK * 2];
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double xp[D];
#pragma unroll
    for (int i = 0; i < D; ++i) xp[i] = p < np ? x[(size_t)p * D + i] : 0.0;
    double tot = 0.0;
    for (int c0 = 0; c0 < nh; c0 += GRF_CHUNK) {
        const int nc = min(GRF_CHUNK, nh - c0);
        __syncthreads();
        for (int i = threadIdx.x; i < nc * D; i += blockDim.x) sk[i] = kappa[(size_t)c0 * D + i];
        for (int i = threadIdx.x; i < nc * 2; i += blockDim.x) sab[i] = ab[(size_t)c0 * 2 + i];
        __syncthreads();
        float part = 0.f;
        for (int k = 0; k < nc; ++k) {
            double ph = 0.0;
#pragma unroll
            for (int i = 0; i < D; ++i) ph = fma(sk[k * D + i], xp[i], ph);
            const double r = fma(-TWO_PI, rint(ph * (1.0 / TWO_PI)), ph);
            float s, c;
            __sincosf((float)r, &s, &c);
            part = fmaf(sab[2 * k], c, part);
            part = fmaf(sab[2 * k + 1], s, part);
        }
        tot += (double)part;
    }
    if (p < np) out[p] = fmax(mean + scale * tot, vmin);
}

}  // namespace ep

using namespace ep;

extern "C" {

ep_status epgpu_grf_spectrum(const ep_grf* g, double* kappa, double* ab) {
    if (!g || !kappa || !ab || (g->dim != 2 && g->dim != 3) || g->nh <= 0 ||
        (g->covariance != EP_GRF_GAUSSIAN && g->covariance != EP_GRF_EXPONENTIAL))
        return EP_ERR_ARG;
    for (int i = 0; i < g->dim; ++i)
        if (!(g->ell[i] > 0.0)) return EP_ERR_ARG;
    grf_spectrum(*g, kappa, ab);
    return EP_OK;
}

ep_status epgpu_grf_points(const ep_grf* g, const double* x, int64_t np, double* out) {
    if (!g || np < 0 || (np > 0 && (!x || !out)) || (g->dim != 2 && g->dim != 3) || g->nh <= 0 ||
        (g->covariance != EP_GRF_GAUSSIAN && g->covariance != EP_GRF_EXPONENTIAL))
        return EP_ERR_ARG;
    for (int i = 0; i < g->dim; ++i)
        if (!(g->ell[i] > 0.0)) return EP_ERR_ARG;
    if (np == 0) return EP_OK;
    const int d = g->dim;
    std::vector<double> kap((size_t)g->nh * d), ab((size_t)g->nh * 2);
    grf_spectrum(*g, kap.data(), ab.data());
    std::vector<float> abf(ab.begin(), ab.end());
    double *dk = nullptr, *dx = nullptr, *dout = nullptr;
    float* dab = nullptr;
    cudaError_t e = cudaMalloc(&dk, kap.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dab, abf.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&dx, (size_t)np * d * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dout, (size_t)np * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(dk, kap.data(), kap.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dab, abf.data(), abf.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, (size_t)np * d * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const double scale = g->std / std::sqrt((double)g->nh);
        const unsigned nb = (unsigned)((np + 255) / 256);
        if (d == 2) k_grf<2><<<nb, 256>>>(dk, dab, g->nh, dx, np, scale, g->mean, g->vmin, dout);
        else k_grf<3><<<nb, 256>>>(dk, dab, g->nh, dx, np, scale, g->mean, g->vmin, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, (size_t)np * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(dk);
    cudaFree(dab);
    cudaFree(dx);
    cudaFree(dout);
    if (e != cudaSuccess) {
        set_global_error((std::string("grf: ") + cudaGetErrorString(e)).c_str());
        cudaGetLastError();
        return EP_ERR_CUDA;
    }
    return EP_OK;
}

}  // extern "C"
